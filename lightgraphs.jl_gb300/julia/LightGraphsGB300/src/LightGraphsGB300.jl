"""
    LightGraphsGB300

GB300 (sm_103a) drop-in for LightGraphs' unit-weight betweenness centrality and
gdistances.  The functions below take the same arguments as

  betweenness_centrality(g[, vs][, distmx]; normalize, endpoints)   src/centrality/betweenness.jl:46-75
  betweenness_centrality(g, k[, distmx]; normalize, endpoints)      src/centrality/betweenness.jl:77-78
  gdistances!(g, source, dists), gdistances(g, source)              src/traversals/bfs.jl:95-141
  Parallel.betweenness_centrality(...; parallel)                    src/Parallel/centrality/betweenness.jl:1-75
  Parallel.gdistances[!](g, source(s)[, dists])                     src/Parallel/traversals/gdistances.jl:36-139
  stress_centrality(g[, vs | k])                                    src/centrality/stress.jl:33-49
  closeness_centrality(g[, distmx]; normalize)                      src/centrality/closeness.jl:33-55
  radiality_centrality(g)                                           src/centrality/radiality.jl:36-49
  eccentricity(g[, v | vs][, distmx])                               src/distance.jl:73-84
  bfs_parents(g, s; dir), bfs_tree(g, s; dir), has_path(g, u, v)    src/traversals/bfs.jl:35-76,150-172
  core_number(g)                                                    src/degeneracy.jl:38-80

restricted to `SimpleGraph` / `SimpleDiGraph` with unit weights (`DefaultDistance`);
another distance matrix is a `MethodError`.  The graph's `fadjlist` (and
`badjlist`) is flattened once to a 0-based Int64/Int32 CSR, uploaded through
`lgbc_graph_create`, and cached per graph object; the work runs in the CUDA
library `liblgbc.so` (C ABI: include/lgbc.h).  Source sampling
(`LightGraphs.sample`) and `LightGraphs._rescale!` stay on the host and are
called unchanged, so their semantics are the reference's by construction.
There is no CPU fallback: without a GPU every call throws.
"""
module LightGraphsGB300

using LightGraphs
using LightGraphs: AbstractGraph, SimpleGraph, SimpleDiGraph, DefaultDistance, nv, ne,
                   is_directed, vertices, weights, degree
using Libdl

export betweenness_centrality, gdistances, gdistances!, stress_centrality, closeness_centrality,
       radiality_centrality, eccentricity, bfs_parents, bfs_tree, has_path, core_number,
       path_counts

const LGBC_OK = Cint(0)
const LGBC_EINVAL = Cint(-1)
const LIB = Ref{Ptr{Cvoid}}(C_NULL)
const SYM = Dict{Symbol,Ptr{Cvoid}}()

function __init__()
    path = get(ENV, "LGBC_LIB", normpath(joinpath(@__DIR__, "..", "..", "..", "lib", "liblgbc.so")))
    LIB[] = Libdl.dlopen(path)
    for s in (:lgbc_graph_create, :lgbc_graph_destroy, :lgbc_gdistances, :lgbc_betweenness,
              :lgbc_last_error, :lgbc_stress, :lgbc_distance_stats, :lgbc_bfs_parents,
              :lgbc_has_path, :lgbc_core_number, :lgbc_tune, :lgbc_path_counts)
        SYM[s] = Libdl.dlsym(LIB[], s)
    end
end

struct LGBCError <: Exception
    code::Cint
    msg::String
end
Base.showerror(io::IO, e::LGBCError) = print(io, "lgbc error ", e.code, ": ", e.msg)

function check(rc::Cint)
    rc == LGBC_OK && return nothing
    msg = unsafe_string(ccall(SYM[:lgbc_last_error], Cstring, ()))
    rc == LGBC_EINVAL && throw(ArgumentError(msg))
    throw(LGBCError(rc, msg))
end

# ---------------------------------------------------------------- device graphs
mutable struct DeviceGraph
    ptr::Ptr{Cvoid}
    fp::UInt64   # fingerprint of the adjacency lists the device copy was built from
    function DeviceGraph(ptr, fp)
        d = new(ptr, fp)
        finalizer(d) do x
            x.ptr != C_NULL && ccall(SYM[:lgbc_graph_destroy], Cint, (Ptr{Cvoid},), x.ptr)
            x.ptr = C_NULL
        end
        return d
    end
end

"""Flatten `adj` (sorted neighbour lists, 1-based) to a 0-based CSR."""
function flatten(adj::Vector{Vector{T}}) where {T<:Integer}
    n = length(adj)
    rowptr = Vector{Int64}(undef, n + 1)
    rowptr[1] = 0
    @inbounds for v in 1:n
        rowptr[v+1] = rowptr[v] + length(adj[v])
    end
    colidx = Vector{Int32}(undef, rowptr[end])
    k = 1
    @inbounds for v in 1:n, u in adj[v]
        colidx[k] = Int32(u - 1)
        k += 1
    end
    return rowptr, colidx
end

"""A 64-bit fingerprint of every (vertex, neighbour) entry of `adj`: any
add_edge! / rem_edge! sequence that leaves the lists different changes it
(up to 64-bit collisions), including edits that keep ne(g) the same."""
function fingerprint(adj::Vector{Vector{T}}) where {T<:Integer}
    h = UInt64(length(adj))
    @inbounds for v in eachindex(adj)
        l = adj[v]
        h = (h ⊻ UInt64(length(l))) * 0x100000001b3
        for u in l
            x = (UInt64(v) << 32) ⊻ UInt64(u)
            x = (x ⊻ (x >> 33)) * 0xff51afd7ed558ccd
            h = (h + (x ⊻ (x >> 29))) * 0x9e3779b97f4a7c15
        end
    end
    return h
end

const CACHE = WeakKeyDict{AbstractGraph,DeviceGraph}()
const CACHE_LOCK = ReentrantLock()

function device_graph(g::Union{SimpleGraph,SimpleDiGraph})
    lock(CACHE_LOCK) do
        fp = fingerprint(g.fadjlist)
        d = get(CACHE, g, nothing)
        d !== nothing && d.fp == fp && return d
        rowptr, colidx = flatten(g.fadjlist)
        dir = is_directed(g)
        in_rowptr, in_colidx = dir ? flatten(g.badjlist) : (Int64[], Int32[])
        out = Ref{Ptr{Cvoid}}(C_NULL)
        GC.@preserve rowptr colidx in_rowptr in_colidx begin
            check(ccall(SYM[:lgbc_graph_create], Cint,
                        (Ptr{Ptr{Cvoid}}, Int64, Int64, Ptr{Int64}, Ptr{Int32}, Ptr{Int64},
                         Ptr{Int32}, Cint),
                        out, nv(g), length(colidx), rowptr, colidx,
                        dir ? pointer(in_rowptr) : C_NULL, dir ? pointer(in_colidx) : C_NULL,
                        Cint(dir)))
        end
        d = DeviceGraph(out[], fp)
        CACHE[g] = d
        return d
    end
end

function sources0(g, vs)
    src = Vector{Int32}(undef, length(vs))
    for (i, v) in enumerate(vs)
        1 <= v <= nv(g) || throw(BoundsError(vertices(g), v))
        src[i] = Int32(v - 1)
    end
    return src
end

# ---------------------------------------------------------------- betweenness
"""
    betweenness_centrality(g[, vs][, distmx]; normalize=true, endpoints=false)
    betweenness_centrality(g, k[, distmx]; normalize=true, endpoints=false)

GPU drop-in for `LightGraphs.betweenness_centrality` with unit weights.
"""
function betweenness_centrality(g::Union{SimpleGraph,SimpleDiGraph}, vs=vertices(g),
                                distmx::DefaultDistance=weights(g);
                                normalize=true, endpoints=false)
    n = nv(g)
    k = length(vs)
    src = sources0(g, vs)
    raw = Vector{Float64}(undef, n)
    if n > 0
        d = device_graph(g)
        GC.@preserve src raw begin
            check(ccall(SYM[:lgbc_betweenness], Cint,
                        (Ptr{Cvoid}, Ptr{Int32}, Int64, Cint, Ptr{Float64}),
                        d.ptr, src, length(src), Cint(endpoints), raw))
        end
    end
    LightGraphs._rescale!(raw, n, normalize, is_directed(g), k)
    return raw
end

betweenness_centrality(g::Union{SimpleGraph,SimpleDiGraph}, k::Integer,
                       distmx::DefaultDistance=weights(g); normalize=true, endpoints=false) =
    betweenness_centrality(g, LightGraphs.sample(vertices(g), k), distmx;
                           normalize=normalize, endpoints=endpoints)

# ---------------------------------------------------------------- gdistances
function device_levels(g, source)
    src = sources0(g, source isa Integer ? [source] : source)
    lv = Vector{Int32}(undef, nv(g))
    if nv(g) > 0
        d = device_graph(g)
        GC.@preserve src lv begin
            check(ccall(SYM[:lgbc_gdistances], Cint, (Ptr{Cvoid}, Ptr{Int32}, Int64, Ptr{Int32}),
                        d.ptr, src, length(src), lv))
        end
    end
    return lv
end

"""
    gdistances!(g, source, vert_level)

GPU drop-in for `LightGraphs.gdistances!`: writes the level of every vertex the
BFS reaches and leaves the other entries untouched.
"""
function gdistances!(g::Union{SimpleGraph{T},SimpleDiGraph{T}}, source, vert_level;
                     sort_alg=nothing) where {T}
    lv = device_levels(g, source)
    @inbounds for v in eachindex(lv)
        lv[v] != typemax(Int32) && (vert_level[v] = T(lv[v]))
    end
    return vert_level
end

"""
    gdistances(g, source)

GPU drop-in for `LightGraphs.gdistances`; unreachable vertices get `typemax(T)`.
"""
gdistances(g::Union{SimpleGraph{T},SimpleDiGraph{T}}, source; sort_alg=nothing) where {T} =
    gdistances!(g, source, fill(typemax(T), nv(g)))

# ---------------------------------------------------------------- stress
"""
    stress_centrality(g[, vs])
    stress_centrality(g, k)

GPU drop-in for `LightGraphs.stress_centrality` (Int64, wrapping like the reference).
"""
function stress_centrality(g::Union{SimpleGraph,SimpleDiGraph}, vs=vertices(g))
    src = sources0(g, vs)
    out = zeros(Int64, nv(g))
    if nv(g) > 0
        d = device_graph(g)
        GC.@preserve src out begin
            check(ccall(SYM[:lgbc_stress], Cint, (Ptr{Cvoid}, Ptr{Int32}, Int64, Ptr{Int64}),
                        d.ptr, src, length(src), out))
        end
    end
    return out
end
stress_centrality(g::Union{SimpleGraph,SimpleDiGraph}, k::Integer) =
    stress_centrality(g, LightGraphs.sample(vertices(g), k))

# ---------------------------------------------------------------- path counts
"""
    path_counts(g, sources) -> (pathcounts, dists)

`dijkstra_shortest_paths(g, s).pathcounts` and `.dists` with unit weights
(src/shortestpaths/dijkstra.jl:59-141) for every `s` in `sources`, as
`nv(g) x length(sources)` matrices (column `i` for `sources[i]`): counts as
Float64 (exact below 2^53), `typemax(T)` distances where `s` does not reach.
"""
function path_counts(g::Union{SimpleGraph{T},SimpleDiGraph{T}}, sources) where {T}
    src = sources0(g, sources)
    pc = zeros(Float64, nv(g), length(src))
    lv = Matrix{Int32}(undef, nv(g), length(src))
    if nv(g) > 0 && !isempty(src)
        d = device_graph(g)
        GC.@preserve src pc lv begin
            check(ccall(SYM[:lgbc_path_counts], Cint,
                        (Ptr{Cvoid}, Ptr{Int32}, Int64, Ptr{Float64}, Ptr{Int32}),
                        d.ptr, src, length(src), pc, lv))
        end
    else
        fill!(lv, typemax(Int32))
    end
    dists = T[l == typemax(Int32) ? typemax(T) : T(l) for l in lv]
    return pc, dists
end

# ---------------------------------------------------------------- distance reductions
"""(reachable count incl. the source, distance sum, largest distance) per source."""
function distance_stats(g, vs)
    src = sources0(g, vs)
    k = length(src)
    reached = Vector{Int64}(undef, k); dsum = Vector{Int64}(undef, k); dmax = Vector{Int32}(undef, k)
    if k > 0
        d = device_graph(g)
        GC.@preserve src reached dsum dmax begin
            check(ccall(SYM[:lgbc_distance_stats], Cint,
                        (Ptr{Cvoid}, Ptr{Int32}, Int64, Ptr{Int64}, Ptr{Int64}, Ptr{Int32}),
                        d.ptr, src, k, reached, dsum, dmax))
        end
    end
    return reached, dsum, dmax
end

"""GPU drop-in for `LightGraphs.closeness_centrality` with unit weights."""
function closeness_centrality(g::Union{SimpleGraph,SimpleDiGraph},
                              distmx::DefaultDistance=weights(g); normalize=true)
    n_v = nv(g)
    closeness = zeros(n_v)
    act = [u for u in vertices(g) if degree(g, u) > 0]
    reached, dsum, _ = distance_stats(g, act)
    for (i, u) in enumerate(act)
        σ = dsum[i]; l = reached[i] - 1
        if σ > 0
            closeness[u] = l / σ
            normalize && (closeness[u] *= l / (n_v - 1))
        end
    end
    return closeness
end

"""GPU drop-in for `LightGraphs.radiality_centrality` (Int64 sums over typemax distances)."""
function radiality_centrality(g::Union{SimpleGraph,SimpleDiGraph})::Vector{Float64}
    n_v = nv(g)
    reached, dsum, dmax = distance_stats(g, vertices(g))
    meandists = zeros(Float64, n_v)
    dmtr = 0.0
    for v in 1:n_v
        unreached = n_v - reached[v]
        dmtr = max(dmtr, unreached > 0 ? typemax(Int) : Int(dmax[v]))
        meandists[v] = (dsum[v] + unreached * typemax(Int)) / (n_v - 1)
    end
    meandists = (dmtr + 1) .- (meandists)
    return meandists ./ dmtr
end

"""GPU drop-in for `LightGraphs.eccentricity` with unit weights."""
function eccentricity(g::Union{SimpleGraph,SimpleDiGraph}, vs=vertices(g),
                      distmx::DefaultDistance=weights(g))
    reached, _, dmax = distance_stats(g, vs)
    e = [reached[i] < nv(g) ? typemax(Int) : Int(dmax[i]) for i in eachindex(reached)]
    any(==(typemax(Int)), e) && @warn("Infinite path length detected")
    return e
end
eccentricity(g::Union{SimpleGraph,SimpleDiGraph}, v::Integer, distmx::DefaultDistance=weights(g)) =
    eccentricity(g, [v], distmx)[1]

# ---------------------------------------------------------------- BFS trees
"""GPU drop-in for `LightGraphs.bfs_parents` (the serial function's parents)."""
function bfs_parents(g::Union{SimpleGraph{T},SimpleDiGraph{T}}, s::Integer; dir=:out) where {T}
    1 <= s <= nv(g) || throw(BoundsError(vertices(g), s))
    p = Vector{Int32}(undef, nv(g))
    d = device_graph(g)
    GC.@preserve p begin
        check(ccall(SYM[:lgbc_bfs_parents], Cint, (Ptr{Cvoid}, Int32, Cint, Ptr{Int32}),
                    d.ptr, Int32(s - 1), Cint(dir == :out ? 0 : 1), p))
    end
    return T[x + 1 for x in p]
end
bfs_tree(g::Union{SimpleGraph,SimpleDiGraph}, s::Integer; dir=:out) =
    LightGraphs.tree(bfs_parents(g, s; dir=dir))

"""GPU drop-in for `LightGraphs.has_path`."""
function has_path(g::Union{SimpleGraph,SimpleDiGraph}, u::Integer, v::Integer;
                  exclude_vertices::AbstractVector=Int[])
    ex = sources0(g, exclude_vertices)
    r = Ref{Cint}(0)
    d = device_graph(g)
    GC.@preserve ex begin
        check(ccall(SYM[:lgbc_has_path], Cint, (Ptr{Cvoid}, Int32, Int32, Ptr{Int32}, Int64, Ref{Cint}),
                    d.ptr, Int32(u - 1), Int32(v - 1), ex, length(ex), r))
    end
    return r[] != 0
end

"""GPU drop-in for `LightGraphs.core_number`."""
function core_number(g::Union{SimpleGraph{T},SimpleDiGraph{T}}) where {T}
    c = Vector{Int32}(undef, nv(g))
    d = device_graph(g)
    GC.@preserve c begin
        check(ccall(SYM[:lgbc_core_number], Cint, (Ptr{Cvoid}, Ptr{Int32}), d.ptr, c))
    end
    return T.(c)
end

"""Run the library's autotuner for `g` (optionally with a cache file)."""
tune!(g::Union{SimpleGraph,SimpleDiGraph}; cache::Union{Nothing,String}=nothing) =
    check(ccall(SYM[:lgbc_tune], Cint, (Ptr{Cvoid}, Cstring), device_graph(g).ptr,
                cache === nothing ? C_NULL : cache))

module Parallel
using ..LightGraphsGB300: LightGraphsGB300, DefaultDistance
using LightGraphs: SimpleGraph, SimpleDiGraph, vertices, weights, nv

"""Parallel.betweenness_centrality: the `parallel` keyword selects nothing on one GPU."""
betweenness_centrality(g::Union{SimpleGraph,SimpleDiGraph}, vs=vertices(g),
                       distmx::DefaultDistance=weights(g); normalize=true, endpoints=false,
                       parallel=:distributed) =
    LightGraphsGB300.betweenness_centrality(g, vs, distmx; normalize=normalize, endpoints=endpoints)

betweenness_centrality(g::Union{SimpleGraph,SimpleDiGraph}, k::Integer,
                       distmx::DefaultDistance=weights(g); normalize=true, endpoints=false,
                       parallel=:distributed) =
    LightGraphsGB300.betweenness_centrality(g, k, distmx; normalize=normalize, endpoints=endpoints)

gdistances(g::Union{SimpleGraph{T},SimpleDiGraph{T}}, sources; queue_segment_size=20) where {T} =
    LightGraphsGB300.gdistances(g, sources)

function gdistances!(g::Union{SimpleGraph{T},SimpleDiGraph{T}}, sources, vert_level;
                     queue_segment_size=20) where {T}
    fill!(vert_level, typemax(T))
    return LightGraphsGB300.gdistances!(g, sources, vert_level)
end

stress_centrality(g::Union{SimpleGraph,SimpleDiGraph}, vs=vertices(g); parallel=:distributed) =
    LightGraphsGB300.stress_centrality(g, vs)
stress_centrality(g::Union{SimpleGraph,SimpleDiGraph}, k::Integer; parallel=:distributed) =
    LightGraphsGB300.stress_centrality(g, k)
closeness_centrality(g::Union{SimpleGraph,SimpleDiGraph}, distmx::DefaultDistance=weights(g);
                     normalize=true, parallel=:distributed) =
    LightGraphsGB300.closeness_centrality(g, distmx; normalize=normalize)
radiality_centrality(g::Union{SimpleGraph,SimpleDiGraph}; parallel=:distributed) =
    LightGraphsGB300.radiality_centrality(g)
eccentricity(g::Union{SimpleGraph,SimpleDiGraph}, vs=vertices(g), distmx::DefaultDistance=weights(g)) =
    LightGraphsGB300.eccentricity(g, vs, distmx)
bfs_tree(g::Union{SimpleGraph,SimpleDiGraph}, s::Integer) = LightGraphsGB300.bfs_tree(g, s)
end # module Parallel

end # module
