"""CPU oracle for the GB300 betweenness / BFS path -- test infrastructure only.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline arm,
never by the product package."""
