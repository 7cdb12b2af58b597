"""The bench's reference arm on CPU: it times the oracle (the reference's
algorithm restated) on the workload's own graph and sources, and the process
never maps the CUDA library -- its graph comes from the oracle's copy of the
generators, and `sample` is plain Python."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CODE = """
import sys
sys.argv = ['bench.py', '--impl', 'reference', '--scale', '12', '--k', '64', '--steps', '1',
            '--warmup', '1']
import bench
bench.main()
maps = open('/proc/self/maps').read()
print('MAPPED', sorted({l.split()[-1].rsplit('/', 1)[-1] for l in maps.splitlines()
                         if l.split()[-1].endswith('.so') and 'lg' in l.split()[-1]}))
"""


def test_reference_arm_maps_no_product_library():
    out = subprocess.run([sys.executable, "-c", CODE], cwd=ROOT, capture_output=True, text=True,
                         timeout=600, check=True).stdout.splitlines()
    line = json.loads(next(l for l in out if l.startswith("{")))
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["config"]["workload"] == "rmat12_sampled_bc_k64"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    mapped = next(l for l in out if l.startswith("MAPPED"))
    assert "liblgbc.so" not in mapped and "liblgoracle.so" in mapped


def test_reference_workload_is_the_gpu_workload():
    # the oracle's generator copy and the library's give the same graph and sources
    sys.path.insert(0, ROOT)
    import types
    import numpy as np
    import bench
    args = types.SimpleNamespace(workload="c2", scale=11, k=100)
    g, src, name = bench.reference_workload(args)
    g2, src2, k_act, _, name2 = bench.workload(0, args)
    assert name == name2 and np.array_equal(src, src2)
    assert np.array_equal(g.csr()[0], g2.csr()[0]) and np.array_equal(g.csr()[1], g2.csr()[1])
