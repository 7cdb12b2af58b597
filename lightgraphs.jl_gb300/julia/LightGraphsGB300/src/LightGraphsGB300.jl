"""
    LightGraphsGB300

GB300 (sm_103a) drop-in for LightGraphs' unit-weight betweenness centrality and
gdistances.  The functions below take the same arguments as

  betweenness_centrality(g[, vs][, distmx]; normalize, endpoints)   src/centrality/betweenness.jl:46-75
  betweenness_centrality(g, k[, distmx]; normalize, endpoints)      src/centrality/betweenness.jl:77-78
  gdistances!(g, source, dists), gdistances(g, source)              src/traversals/bfs.jl:95-141
  Parallel.betweenness_centrality(...; parallel)                    src/Parallel/centrality/betweenness.jl:1-75
  Parallel.gdistances[!](g, source(s)[, dists])                     src/Parallel/traversals/gdistances.jl:36-139

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

export betweenness_centrality, gdistances, gdistances!

const LGBC_OK = Cint(0)
const LGBC_EINVAL = Cint(-1)
const LIB = Ref{Ptr{Cvoid}}(C_NULL)
const SYM = Dict{Symbol,Ptr{Cvoid}}()

function __init__()
    path = get(ENV, "LGBC_LIB", normpath(joinpath(@__DIR__, "..", "..", "..", "lib", "liblgbc.so")))
    LIB[] = Libdl.dlopen(path)
    for s in (:lgbc_graph_create, :lgbc_graph_destroy, :lgbc_gdistances, :lgbc_betweenness,
              :lgbc_last_error)
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
    ne::Int
    function DeviceGraph(ptr, ne)
        d = new(ptr, ne)
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

const CACHE = WeakKeyDict{AbstractGraph,DeviceGraph}()
const CACHE_LOCK = ReentrantLock()

function device_graph(g::Union{SimpleGraph,SimpleDiGraph})
    lock(CACHE_LOCK) do
        d = get(CACHE, g, nothing)
        d !== nothing && d.ne == ne(g) && return d
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
        d = DeviceGraph(out[], ne(g))
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
end # module Parallel

end # module
