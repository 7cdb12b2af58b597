"""Regenerate the golden fixtures in this folder from the reference's own test data.

Run from the repository root in a checkout that has the LightGraphs.jl v1.3.5
sources next to it:

    python tests/golden/make_golden.py <path to the LightGraphs.jl v1.3.5 checkout>

It copies, in plain text, the reference's golden graph and vectors:
  * test/testdata/graph-50-500.jgz     -> graph-50-500.lg   (gunzipped LG format)
  * test/testdata/graph-50-500-bc.txt  -> graph-50-500-bc.txt (betweenness, normalize=true)
  * test/testdata/graph-50-500-sc.txt  -> graph-50-500-sc.txt (stress centrality)
  * test/testdata/graph-50-500-rc.txt  -> graph-50-500-rc.txt (radiality centrality)
  * test/testdata/graph-decomposition.jgz -> graph-decomposition.lg (core numbers,
    test/degeneracy.jl:2-6)
and writes ``known_answers.json``: the small known-answer cases that the
reference's tests assert (each entry carries the test file:line it restates).
Nothing at test time reads the reference tree; the tests only read this folder.
"""
import gzip
import json
import os
import shutil
import sys


def main(ref_root: str) -> None:
    here = os.path.dirname(os.path.abspath(__file__))
    td = os.path.join(ref_root, "test", "testdata")
    with gzip.open(os.path.join(td, "graph-50-500.jgz"), "rt") as f:
        text = f.read()
    with open(os.path.join(here, "graph-50-500.lg"), "w") as f:
        f.write(text)
    for suffix in ("bc", "sc", "rc"):
        shutil.copyfile(os.path.join(td, f"graph-50-500-{suffix}.txt"),
                        os.path.join(here, f"graph-50-500-{suffix}.txt"))
    with gzip.open(os.path.join(td, "graph-decomposition.jgz"), "rt") as f:
        text = f.read()
    with open(os.path.join(here, "graph-decomposition.lg"), "w") as f:
        f.write(text)

    # Known answers asserted by the reference's tests (1-based vertex ids).
    known = {
        "betweenness": [
            {"cite": "test/centrality/betweenness.jl:2-5,28",
             "name": "s1 = SimpleGraph(s2)", "n": 3, "directed": False,
             "edges": [[1, 2], [2, 3], [3, 3]], "normalize": True, "endpoints": False,
             "expected": [0.0, 1.0, 0.0]},
            {"cite": "test/centrality/betweenness.jl:2-5,29",
             "name": "s2 (1->2->3, 3->3)", "n": 3, "directed": True,
             "edges": [[1, 2], [2, 3], [3, 3]], "normalize": True, "endpoints": False,
             "expected": [0.0, 0.5, 0.0]},
            {"cite": "test/centrality/betweenness.jl:31-37",
             "name": "2-vertex graph", "n": 2, "directed": False,
             "edges": [[1, 2]], "normalize": True, "endpoints": False,
             "expected": [0.0, 0.0]},
            {"cite": "src/centrality/betweenness.jl:32-36 (doc example)",
             "name": "star_graph(3)", "n": 3, "directed": False,
             "edges": [[1, 2], [1, 3]], "normalize": True, "endpoints": False,
             "expected": [1.0, 0.0, 0.0]},
            {"cite": "src/centrality/betweenness.jl:38-43 (doc example)",
             "name": "path_graph(4)", "n": 4, "directed": False,
             "edges": [[1, 2], [2, 3], [3, 4]], "normalize": True, "endpoints": False,
             "expected": [0.0, 0.6666666666666666, 0.6666666666666666, 0.0]},
        ],
        "betweenness_partial": [
            {"cite": "test/centrality/betweenness.jl:6,40-41",
             "name": "path_graph(5), normalize=false: endpoints of the path are 0",
             "n": 5, "directed": False, "edges": [[1, 2], [2, 3], [3, 4], [4, 5]],
             "normalize": False, "endpoints": False, "zero_at": [1, 5]},
        ],
        "golden_endpoints": {
            "cite": "test/centrality/betweenness.jl:15-17",
            "graph": "graph-50-500", "normalize": False, "endpoints": True,
            "first3": [122.10760591498584, 159.0072453120582, 176.39547945994505],
            "digits": 4},
        "core_number": {
            "cite": "test/degeneracy.jl:2-6", "graph": "graph-decomposition",
            "expected": [3, 3, 3, 3, 3, 3, 3, 3, 2, 2, 2, 2, 2, 2, 2, 2, 1, 1, 1, 1, 0]},
        "dijkstra": [
            {"cite": "test/shortestpaths/dijkstra.jl:77-93",
             "n": 5, "directed": False,
             "edges": [[1, 2], [1, 3], [2, 5], [3, 5], [3, 4], [4, 5]], "source": 1,
             "pathcounts": [1.0, 1.0, 1.0, 1.0, 2.0],
             "predecessors": [[], [1], [1], [3], [2, 3]],
             "closest_vertices": [1, 2, 3, 5, 4]},
            {"cite": "test/shortestpaths/dijkstra.jl:95-103",
             "n": 5, "directed": False, "edges": [[1, 2], [1, 3], [4, 5]], "source": 1,
             "closest_vertices": [1, 2, 3, 4, 5]},
        ],
        "gdistances": [
            {"cite": "test/traversals/bfs.jl:6,29-35 (smallgraph(:house),"
                     " src/SimpleGraphs/generators/smallgraphs.jl:202-205)",
             "n": 5, "directed": False,
             "edges": [[1, 2], [1, 3], [2, 4], [3, 4], [3, 5], [4, 5]],
             "cases": [{"sources": [2], "expected": [1, 0, 2, 1, 2]},
                       {"sources": [1, 2], "expected": [0, 0, 1, 1, 2]},
                       {"sources": [], "expected": ["typemax"] * 5}]},
            {"cite": "test/parallel/traversals/gdistances.jl:4-10 (g5 digraph;"
                     " expected values are the serial gdistances result)",
             "n": 4, "directed": True, "edges": [[1, 2], [2, 3], [1, 3], [3, 4]],
             "cases": [{"sources": [1], "expected": [0, 1, 1, 2]},
                       {"sources": [1, 3], "expected": [0, 1, 0, 1]}]},
        ],
    }
    with open(os.path.join(here, "known_answers.json"), "w") as f:
        json.dump(known, f, indent=1)
    print("wrote fixtures to", here)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path to the LightGraphs.jl checkout>")
    main(sys.argv[1])
