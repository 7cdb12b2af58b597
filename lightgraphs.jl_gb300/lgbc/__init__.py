"""lgbc -- GB300-native betweenness centrality and BFS for LightGraphs graphs.

A host-side mirror of the LightGraphs.jl v1.3.5 interface for this path
(1-based vertex ids, the same names, keywords and exceptions), calling the
CUDA library ``liblgbc.so`` through its C ABI (include/lgbc.h):

    betweenness_centrality(g[, vs | k][, distmx]; normalize, endpoints)
        src/centrality/betweenness.jl:46-78
    Parallel.betweenness_centrality(...; parallel)
        src/Parallel/centrality/betweenness.jl:1-75
    gdistances(g, s | sources), gdistances_(g, s, dists)  (Julia's gdistances!)
        src/traversals/bfs.jl:95-141
    Parallel.gdistances / Parallel.gdistances_
        src/Parallel/traversals/gdistances.jl:36-139

    stress_centrality(g[, vs | k])                  src/centrality/stress.jl:33-49
    bfs_parents, bfs_tree, tree, has_path           src/traversals/bfs.jl:10-76,150-172
    path_counts(g, sources) -- dijkstra_shortest_paths(g, s).pathcounts / .dists
                                                    src/shortestpaths/dijkstra.jl:59-141
    core_number(g)                                  src/degeneracy.jl:38-80
    closeness_centrality, radiality_centrality      src/centrality/{closeness,radiality}.jl
    eccentricity, diameter, radius, periphery, center  src/distance.jl:73-170
    learned.* -- importance-sampled betweenness with a learned source
        proposal (no counterpart in the reference)

Graphs are ``SimpleGraph`` / ``SimpleDiGraph`` (CSR-backed mirrors of
LightGraphs' fadjlist storage).  Every computation runs on the GPU; without
a GPU or without the built library the calls raise ``LGBCError``.
"""
from . import Parallel, learned
from ._lib import ArgumentError, BoundsError, LGBCError, MethodError
from .centrality import (betweenness_centrality, betweenness_centrality_many, betweenness_raw,
                         sample, sample_, stress_centrality, _rescale_)
from .graphs import (DefaultDistance, DeviceGraph, SimpleDiGraph, SimpleGraph, degree,
                     graph_from_edges, is_directed, ne, nv, vertices, weights)
from .persistence import loadgraph
from .distance import (center, closeness_centrality, diameter, eccentricity, periphery,
                       radiality_centrality, radius)
from .learned import (SourceProposal, betweenness_centrality_learned, core_number,
                      dependency_mass, features)
from .traversals import (bfs_parents, bfs_tree, gdistances, gdistances_, has_path,
                         multi_gdistances, path_counts, tree)

__all__ = [
    "Parallel", "ArgumentError", "BoundsError", "LGBCError", "MethodError",
    "betweenness_centrality", "betweenness_centrality_many", "betweenness_raw", "sample", "sample_", "_rescale_",
    "DefaultDistance", "DeviceGraph", "SimpleDiGraph", "SimpleGraph", "degree", "is_directed",
    "ne", "nv", "vertices", "weights", "loadgraph", "gdistances", "gdistances_",
    "multi_gdistances", "learned", "SourceProposal", "betweenness_centrality_learned",
    "core_number", "dependency_mass", "features", "closeness_centrality", "radiality_centrality",
    "eccentricity", "diameter", "radius", "periphery", "center", "stress_centrality",
    "bfs_parents", "bfs_tree", "tree", "has_path", "graph_from_edges", "path_counts",
]
