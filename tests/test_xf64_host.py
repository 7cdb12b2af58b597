"""The extended-precision dependency arithmetic (csrc/xf64.cuh) on the host.

The dependency sweep computes psi = 1/sigma + sum(psi of successors) and
delta = sigma * sum on the integer pipes in a 64-bit-significand format
(xf64).  These tests compile the same header for the CPU (tests/xf64_check.cpp)
and compare every operation with exact rational arithmetic: each result must
be within 2^-60 of the exact value, i.e. well inside one binary64 rounding
(2^-53), and the binary64 rounding of the result must be the correctly
rounded value or its neighbour.
"""
import os
import shutil
import struct
import subprocess
import tempfile
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "lightgraphs.jl_gb300", "csrc")
BIAS = 1085


@pytest.fixture(scope="module")
def harness():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    d = tempfile.mkdtemp(prefix="xf64_")
    exe = os.path.join(d, "xf64_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-w", "-I", CSRC, "-o", exe,
                    os.path.join(ROOT, "tests", "xf64_check.cpp")], check=True)
    yield exe
    shutil.rmtree(d, ignore_errors=True)


def run(exe, lines):
    out = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True,
                         check=True).stdout.split("\n")
    res = []
    for ln in out:
        if ln.strip():
            m, e, b = ln.split()
            res.append((int(m), int(e), int(b)))
    return res


def bits(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def from_bits(b: int) -> float:
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def xval(m, e):
    return Fraction(m) * Fraction(2) ** (e - BIAS)


def check(res, exact, rel=2.0 ** -60):
    m, e, b = res
    if exact == 0:
        assert m == 0 and e == 0 and b == 0
        return
    assert (1 << 62) <= m < (1 << 63), m
    got = xval(m, e)
    assert abs(got - exact) <= exact * Fraction(rel), (float(got), float(exact))
    want = float(exact)  # correctly rounded
    d = from_bits(b)
    if rel <= 2.0 ** -55:  # the result rounds to the correct value or its neighbour
        assert d == want or d == np.nextafter(want, np.inf) or d == np.nextafter(want, -np.inf)
    else:  # the rounding of a value within rel of exact
        assert abs(Fraction(d) - exact) <= exact * Fraction(rel) + Fraction(abs(want)) * 2 ** -53
    return d == want


def test_reciprocal_of_path_counts(harness):
    rng = np.random.default_rng(1)
    s = [1, 2, 3, 5, 7, 2**31 - 1, 2**32 + 1, 2**52 + 1, 2**53 - 1, 2**53 + 1, 2**63,
         2**63 + 1, 2**64 - 1, 2**64 - 2**40, 2**63 + 2**40 - 1, 2**63 + 2**40]
    s += [int(x) for x in rng.integers(1, 1000, 200)]
    for k in range(1, 64):
        s += [int(x) for x in rng.integers(2**(k - 1), 2**k, 8, dtype=np.uint64)]
        s += [2**k - 1, 2**k, 2**k + 1]
    s = [x for x in s if 1 <= x < 2**64]
    res = run(harness, [f"R {x}" for x in s])
    exact_round = 0
    for x, r in zip(s, res):
        exact_round += bool(check(r, Fraction(1, x)))
    # a reciprocal within 2^-60 of exact rounds correctly unless it sits that
    # close to a rounding tie (about 2^-8 of the cases)
    assert exact_round >= len(s) - len(s) // 100


def test_product_with_path_counts(harness):
    rng = np.random.default_rng(2)
    lines, exact = [], []
    for _ in range(2000):
        a = float(np.exp(rng.uniform(-60, 40)))
        s = int(rng.integers(1, 2**63, dtype=np.uint64)) >> int(rng.integers(0, 63))
        s = max(s, 1)
        lines.append(f"M {bits(a)} {s}")
        exact.append(Fraction(a) * s)
    for r, ex in zip(run(harness, lines), exact):
        check(r, ex)


def test_add_and_mul(harness):
    rng = np.random.default_rng(3)
    lines, exact = [], []
    for _ in range(2000):
        a = float(np.exp(rng.uniform(-50, 30)))
        b = float(np.exp(rng.uniform(-50, 30))) if rng.random() < 0.9 else 0.0
        lines.append(f"A {bits(a)} {bits(b)}")
        exact.append(Fraction(a) + Fraction(b))
        lines.append(f"X {bits(a)} {bits(b)}")
        exact.append(Fraction(a) * Fraction(b))
    for r, ex in zip(run(harness, lines), exact):
        check(r, ex)


def test_sums_of_many_terms_beat_fp64(harness):
    # the dependency sums: many positive terms of widely different size; the
    # accumulated error stays within (n + 1) 2^-62, far below sequential FP64
    rng = np.random.default_rng(4)
    lines, exact, seq = [], [], []
    for _ in range(300):
        n = int(rng.integers(1, 600))
        xs = [float(np.exp(rng.uniform(-44, 20))) for _ in range(n)]
        lines.append("S %d %s" % (n, " ".join(str(bits(x)) for x in xs)))
        exact.append(sum(Fraction(x) for x in xs))
        acc = 0.0
        for x in xs:
            acc += x
        seq.append(acc)
    ours, fp64 = [], []
    for r, ex, sq, ln in zip(run(harness, lines), exact, seq, lines):
        n = int(ln.split()[1])
        check(r, ex, rel=2.0 ** -62 * (n + 1))  # sequential binary64 allows n 2^-53
        ours.append(float(abs(xval(r[0], r[1]) - ex) / ex))
        fp64.append(float(abs(Fraction(sq) - ex) / ex))
    # before the final rounding the accumulator is far more accurate than a
    # binary64 running sum, and after it no worse on average
    assert np.mean(ours) < np.mean(fp64) / 8
    rounded = [float(abs(Fraction(from_bits(r[2])) - ex) / ex)
               for r, ex in zip(run(harness, lines), exact)]
    assert np.mean(rounded) <= np.mean(fp64)


def test_gather_accumulator(harness):
    # xg64: 58-bit accumulator renormalised every 32 terms (one edge chunk)
    rng = np.random.default_rng(5)
    lines, exact = [], []
    for _ in range(300):
        n = int(rng.integers(1, 300))
        spread = float(rng.choice([1.0, 10.0, 60.0]))
        xs = [float(np.exp(rng.uniform(-spread, spread))) for _ in range(n)]
        lines.append("G %d %s" % (n, " ".join(str(bits(x)) for x in xs)))
        exact.append(sum(Fraction(x) for x in xs))
    for r, ex, ln in zip(run(harness, lines), exact, lines):
        n = int(ln.split()[1])
        # a binary64 running sum is only bounded by n 2^-53
        check(r, ex, rel=2.0 ** -57 * (n + 1))


def test_zero_and_powers_of_two(harness):
    res = run(harness, ["S 0", f"A 0 {bits(1.0)}", "R 1", "R 1024", f"M {bits(0.5)} 1"])
    assert res[0] == (0, 0, 0)
    assert from_bits(res[1][2]) == 1.0
    assert from_bits(res[2][2]) == 1.0
    assert from_bits(res[3][2]) == 1.0 / 1024
    assert from_bits(res[4][2]) == 0.5
