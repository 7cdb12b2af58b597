"""The equal-error comparison behind the learned-proposal workload, on
synthetic records with a known answer: errors falling as c / sqrt(k) and GPU
time linear in k (no GPU involved)."""
import math

import numpy as np
import pytest

from lgbc import compare


def _records(method, ks, c, ms_per_source, seeds=3):
    out = []
    for k in ks:
        for s in range(seeds):
            out.append(dict(method=method, k=k, seed=s, l1=c / math.sqrt(k), top1=0.1,
                            gpu_ms=ms_per_source * k))
    return out


def test_interp_loglog_exact_on_power_laws():
    xs = [256, 1024, 4096, 16384]
    ys = [2.0 / math.sqrt(x) for x in xs]
    for target_x in (300.0, 2000.0, 10000.0):
        assert compare._interp_loglog(xs, ys, 2.0 / math.sqrt(target_x)) == pytest.approx(target_x)
    # beyond the measured budgets the end segments are extended
    assert compare._interp_loglog(xs, ys, 2.0 / math.sqrt(65536)) == pytest.approx(65536)


def test_summarise_equal_error_ratio():
    # learned reaches uniform's error with (0.8)^2 = 0.64 of the sources and
    # costs 1.25x per source, so the equal-error time ratio is 0.8
    ks = [256, 512, 1024, 2048, 4096, 8192, 16384]
    recs = _records("uniform", [1024, 4096, 16384], 1.0, 0.04)
    recs += _records("learned", ks, 0.8, 0.05)
    out = compare.summarise(recs, build_ms=10.0, k_targets=[1024, 4096, 16384])
    for row in out["equal_error"]:
        assert row["k_learned_equal_l1"] == pytest.approx(0.64 * row["k_uniform"])
        assert row["time_ratio"] == pytest.approx(0.8)
        assert row["time_ratio_with_build"] == pytest.approx(0.8 + 10.0 / row["ms_uniform"])
    assert "equal_error_systematic" not in out


def test_means_per_budget():
    recs = [dict(method="uniform", k=8, seed=s, l1=float(s), top1=0.0, gpu_ms=1.0 + s)
            for s in range(4)]
    (row,) = compare._means(recs, "uniform")
    assert row["k"] == 8 and row["l1"] == pytest.approx(1.5)
    assert row["l1_sd"] == pytest.approx(np.std([0, 1, 2, 3]))
    assert row["gpu_ms"] == pytest.approx(2.5)  # median


def test_summarise_ceiling_arms_carry_no_build():
    # a fixed proposal built from exact masses: half the sources at equal
    # error, same cost per source -> ratio 0.5 with and without the build
    ks = [256, 512, 1024, 2048, 4096, 8192, 16384]
    recs = _records("uniform", [1024, 4096, 16384], 1.0, 0.04)
    recs += _records("learned", ks, 0.8, 0.05)
    recs += _records("mass", ks, math.sqrt(0.5), 0.04)
    out = compare.summarise(recs, build_ms=10.0, k_targets=[1024, 4096, 16384],
                            methods=("learned", "mass"))
    for row in out["equal_error_mass"]:
        assert row["k_learned_equal_l1"] == pytest.approx(0.5 * row["k_uniform"])
        assert row["time_ratio"] == pytest.approx(0.5)
        assert row["time_ratio_with_build"] == pytest.approx(0.5)
    assert out["equal_error"][0]["time_ratio_with_build"] > 0.8
