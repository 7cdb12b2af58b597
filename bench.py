#!/usr/bin/env python3
"""Benchmark: sampled Brandes betweenness on an undirected R-MAT scale-20 graph.

Workload (one "step"): betweenness_centrality(g, 4096) on R-MAT scale 20
(n = 2^20, 16 n edge draws, a/b/c/d = .57/.19/.19/.05, self-loops and
duplicates removed, ids permuted; Int32 CSR), sources drawn without
replacement by `sample` (seed 2 + rank).  Sources of degree 0 are skipped, as
in the reference.  Metric: GTEPS = (active sources x undirected edges) / time.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` times K steps with the graph resident
in HBM (CUDA events on the library's stream); `e2e` times the C-ABI call with
host buffers: graph upload from pinned memory, the betweenness call, the
result read back, and the handle freed, every step.  The inputs (CSR 134 MB,
per-batch lane state 1 GB) are larger than the 129 MB L2, so no L2 flush is
inserted.  `--impl reference` times the CPU restatement of the reference
algorithm (heap Dijkstra + predecessor lists, one source per host thread).
"""
from __future__ import annotations

import argparse
import csv
import ctypes
import io
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "lightgraphs.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Brandes BC GTEPS on 1 GB300"
UNIT = "GTEPS"
LANES = 64


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ----------------------------------------------------------------------------- ranks
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ----------------------------------------------------------------------------- clocks
class Clocks:
    """nvidia-smi samples taken every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = os.path.join("/tmp", f"lgbc_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for row in csv.reader(f):
                if len(row) < 9:
                    continue
                try:
                    sm.append(float(row[1]))
                    smax.append(float(row[2]))
                except ValueError:
                    continue
                for nm, val in zip(names, row[5:9]):
                    if val.strip().lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------- helpers
def peak_hbm() -> tuple[float, str]:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def bc_algorithmic_bytes(n: int, nnz: int, k_act: int, lanes: int = LANES) -> int:
    """Brandes bytes for k_act sources in batches of `lanes` sources: per batch
    the CSR is streamed forward and backward and bc read-modified once
    (8 nnz + 32 n + 16 bytes); per source the lane state (write d 4 B + sigma
    8 B, read d 4 B + sigma 8 B, write delta 8 B) is 32 n bytes."""
    return math.ceil(k_act / lanes) * (8 * nnz + 32 * n + 16) + 32 * n * k_act


def gd_algorithmic_bytes(n: int, nnz: int, q: int) -> int:
    return math.ceil(q / LANES) * (4 * nnz + 8 * (n + 1)) + 4 * n * q


def traffic_per_step() -> float | None:
    """DRAM bytes per step from the committed ncu summary, if one exists."""
    p = os.path.join(ROOT, "profiles", "bc_rmat20_k4096_traffic.txt")
    try:
        with open(p) as f:
            for line in f:
                if line.startswith("dram_bytes_per_step:"):
                    return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


WORKLOADS = {
    "c1": "ER G(n=10000, m=50000) undirected, exact BC (all sources)",
    "c2": "R-MAT scale 20 undirected, sampled BC k=4096",
    "c3": "4096 Barabasi-Albert graphs n~U[200,20000], k=3, exact BC for every graph",
    "c4": "R-MAT scale 22 directed, sampled BC k=16384",
    "c5": "learned vs uniform source sampling: R-MAT scale 20 copy and a 10^5-vertex BFS ball "
          "of R-MAT scale 24, k in {1024, 4096, 16384}, 8 seeds",
}


def dep_dtype(tuning: dict) -> str:
    """The arithmetic of the timed path: exact uint64 path counts (FP64 after
    an overflow) and FP64 dependency sums, or double-float ones when the
    dependency_df32 tuning field is set."""
    if int(tuning.get("dependency_df32", 0)):
        return "u64 path counts, df32 dependencies (opt-in, narrower than f64)"
    return "u64 path counts, f64 dependencies"


def parse_tuning(spec: str | None) -> dict:
    """"key=value,..." -> lgbc_tuning overrides (numbers)."""
    out = {}
    for item in (spec or "").split(","):
        if not item.strip():
            continue
        k, v = item.split("=", 1)
        out[k.strip()] = float(v) if k.strip() in ("alpha", "beta") else int(v)
    return out


def workload(rank: int, args):
    """(graph, 0-based sources, active source count, generation seconds, name)."""
    from lgbc import generators as G
    import lgbc
    t = time.perf_counter()
    if args.workload == "c1":
        g = G.erdos_renyi_nm(10000, 50000, seed=1, eltype=np.int64)
        src = np.arange(g.nv(), dtype=np.int32)
        name = "er10k_m50k_exact_bc"
    elif args.workload == "c4":
        g = G.rmat(22, 16, seed=1, directed=True)
        src1 = lgbc.sample(g.vertices(), args.k or 16384, rng=np.random.default_rng(2 + rank))
        src = (np.asarray(src1, np.int64) - 1).astype(np.int32)
        name = f"rmat22_directed_sampled_bc_k{len(src)}"
    else:
        g = G.rmat(args.scale, 16, seed=1)
        src1 = lgbc.sample(g.vertices(), args.k or 4096, rng=np.random.default_rng(2 + rank))
        src = (np.asarray(src1, np.int64) - 1).astype(np.int32)
        name = f"rmat{args.scale}_sampled_bc_k{len(src)}"
    gen_s = time.perf_counter() - t
    deg = g.degrees()
    k_act = int(np.count_nonzero(deg[src] > 0))
    return g, src, k_act, gen_s, name


def one_batch(g, src: np.ndarray, b: int, wname: str):
    """Batch b (128 sources) of the workload as the library batches it: the
    active sources ordered by their BFS distances to the 16 highest-degree
    vertices (ties: smaller id), lexicographically, then by id -- the order
    the source_order tuning gives.  A profiling case of one representative
    batch of the full step."""
    import lgbc
    deg = g.degrees()
    act = src[deg[src] > 0]
    lm = np.lexsort((np.arange(g.nv()), -deg))[:16]
    lm = lm[deg[lm] > 0]
    d = lgbc.multi_gdistances(g, list(lm + 1)).astype(np.int64)[:, act]
    order = np.lexsort((act,) + tuple(d[j] for j in reversed(range(len(lm)))))
    sel = act[order][128 * b:128 * (b + 1)]
    if len(sel) == 0:
        raise SystemExit(f"--profile-batch {b}: the workload has {len(act)} active sources")
    return sel.astype(np.int32), f"{wname}_batch{b}"


def many_graphs(rank: int, count: int, gen=None):
    """Config C3: `count` BA graphs, n uniform in [200, 20000] (seed 0), k = 3,
    graph i seeded 1000 + i.  `gen` is the generator module (the library's by
    default; the CPU arm passes the oracle's, built from the same source)."""
    if gen is None:
        from lgbc import generators as gen
    rng = np.random.default_rng(0 + rank)
    ns = rng.integers(200, 20001, count)
    return [gen.barabasi_albert(int(n), 3, seed=1000 + i) for i, n in enumerate(ns)]


def reference_workload(args):
    """The workload's graph and sources for the CPU arm: the same generator
    source, seeds and `sample` draw as `workload`, built through the oracle's
    copy of the generators so that this arm maps no library of the product."""
    from oracle import oracle
    from lgbc.centrality import sample  # pure Python (src/utils.jl:12-43)
    if args.workload == "c1":
        g = oracle.erdos_renyi_nm(10000, 50000, seed=1)
        return g, np.arange(g.nv(), dtype=np.int32), "er10k_m50k_exact_bc"
    if args.workload == "c4":
        g = oracle.rmat(22, 16, seed=1, directed=True)
        k = args.k or 16384
        name = "rmat22_directed_sampled_bc_k"
    else:
        g = oracle.rmat(args.scale, 16, seed=1)
        k = args.k or 4096
        name = f"rmat{args.scale}_sampled_bc_k"
    src1 = sample(range(1, g.nv() + 1), k, rng=np.random.default_rng(2))
    src = (np.asarray(src1, np.int64) - 1).astype(np.int32)
    return g, src, name + str(len(src))


# ----------------------------------------------------------------------------- CPU arms
def cpu_betweenness_sample(g, src: np.ndarray, nthreads: int, target_s: float, seed: int,
                           mode: str = "faithful"):
    """Time the oracle (mode "faithful": the reference's heap Dijkstra with
    predecessor lists; "fast": BFS Brandes, the same values) on a bounded
    sample of the workload's sources; returns (GTEPS, seconds, sources)."""
    from oracle import oracle
    rp, ci = g.csr()
    kw = {}
    if g.is_directed():
        irp, ici = g.in_csr()
        kw = dict(directed=True, in_rowptr=irp, in_colidx=ici)
    deg = g.degrees()
    act = src[deg[src] > 0]
    rng = np.random.default_rng(seed)
    # calibrate with one source per thread
    cal = rng.choice(act, size=min(len(act), nthreads), replace=False)
    t = time.perf_counter()
    oracle.betweenness_raw(rp, ci, cal, mode=mode, nthreads=nthreads, **kw)
    dt = max(time.perf_counter() - t, 1e-3)
    per_round = dt
    rounds = max(1, int(target_s / per_round))
    count = min(len(act), rounds * nthreads)
    samp = rng.choice(act, size=count, replace=False)
    t = time.perf_counter()
    oracle.betweenness_raw(rp, ci, samp, mode=mode, nthreads=nthreads, **kw)
    dt = time.perf_counter() - t
    m = g.ne()
    return count * m / dt / 1e9, dt, count


def run_reference(args, dist: Dist):
    """--impl reference: the reference's algorithm on the host cores."""
    if dist.rank != 0:
        return
    nthreads = os.cpu_count() or 1
    if args.workload == "c3":
        return run_reference_many(args, nthreads)
    g, src, wname = reference_workload(args)
    rp, ci = g.csr()
    kw = {}
    if g.is_directed():
        irp, ici = g.in_csr()
        kw = dict(directed=True, in_rowptr=irp, in_colidx=ici)
    deg = g.degrees()
    act = src[deg[src] > 0]
    k_act = len(act)
    from oracle import oracle
    m = g.ne()
    per_step = []
    count = None
    for it in range(args.warmup + args.steps):
        if count is None:
            # size one step to about 10 s of CPU work
            cal = act[:nthreads]
            t = time.perf_counter()
            oracle.betweenness_raw(rp, ci, cal, mode="faithful", nthreads=nthreads, **kw)
            dt = max(time.perf_counter() - t, 1e-3)
            count = min(len(act), max(nthreads, int(10.0 / dt) * nthreads))
        samp = act[(it * count) % len(act):][:count]
        if len(samp) < count:
            samp = np.concatenate([samp, act[:count - len(samp)]])
        t = time.perf_counter()
        oracle.betweenness_raw(rp, ci, samp, mode="faithful", nthreads=nthreads, **kw)
        dt = time.perf_counter() - t
        if it >= args.warmup:
            per_step.append(dt)
    t_step = statistics.mean(per_step)
    value = count * m / t_step / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": wname, "n": g.nv(), "m": m, "active_sources": k_act},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": f"{count} of the {k_act} active sources per step "
                                   "(heap Dijkstra + predecessor lists, as "
                                   "src/shortestpaths/dijkstra.jl:59-141; Julia is not "
                                   "installed, so the C++ restatement stands in)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU arm
def run_ours(args, dist: Dist):
    visible = [d for d in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if d.strip()]
    if dist.world > 1:
        # one GPU per rank: rank-local device 0 (set before the library loads)
        mine = visible[dist.local] if len(visible) > dist.local else str(dist.local)
        os.environ["CUDA_VISIBLE_DEVICES"] = mine
        visible = [mine]
    smi_index = int(visible[0]) if visible and visible[0].strip().isdigit() else 0
    import lgbc
    from lgbc import _lib
    lib = _lib.lib()
    if args.workload == "c3":
        return run_ours_many(args, dist)
    g, src, k_act, gen_s, wname = workload(dist.rank, args)
    if args.profile_batch is not None:
        src, wname = one_batch(g, src, args.profile_batch, wname)
        k_act = len(src)
    n, m = g.nv(), g.ne()
    rp, ci = g.csr()
    nnz = len(ci)
    directed = g.is_directed()
    if directed:
        irp, ici = g.in_csr()
    log(f"[rank {dist.rank}] {wname}: n={n} m={m} nnz={nnz} "
        f"sources={len(src)} active={k_act} (generated in {gen_s:.1f}s)")

    dg = g.device_handle()
    h = dg.handle
    overrides = parse_tuning(args.tuning)
    if overrides:
        dg.set_tuning(**overrides)
    tune_s = None
    if args.autotune:
        t0 = time.perf_counter()
        dg.tune()
        tune_s = time.perf_counter() - t0
    tuning = {k: getattr(dg.tuning(), k) for k, _ in _lib.LgbcTuning._fields_}
    log(f"[rank {dist.rank}] tuning {tuning}" + (f" (autotuned in {tune_s:.2f} s)" if tune_s else ""))
    if args.profile_gdistances:
        # only the gdistances calls of the workload (for ncu launch lists):
        # the 64-source batch, then single-source calls from 8 of its sources
        rng = np.random.default_rng(3 + dist.rank)
        gsrc = rng.choice(n, 64, replace=False).astype(np.int32)
        out = np.empty((64, n), np.int32)
        ms = ctypes.c_double()
        _lib.check(lib.lgbc_timer_start(h))
        for _ in range(max(1, args.steps)):
            _lib.check(lib.lgbc_gdistances_batch(h, _lib.ptr(gsrc), 64, _lib.ptr(out)))
        _lib.check(lib.lgbc_timer_stop(h, ctypes.byref(ms), None))
        t_batch = ms.value / max(1, args.steps)
        ss = [np.array([s_], np.int32) for s_ in gsrc[np.diff(rp)[gsrc] > 0][:8]]
        _lib.check(lib.lgbc_timer_start(h))
        for a in ss:
            _lib.check(lib.lgbc_gdistances(h, _lib.ptr(a), 1, _lib.ptr(out[0])))
        _lib.check(lib.lgbc_timer_stop(h, ctypes.byref(ms), None))
        if dist.rank == 0:
            print(json.dumps({"profile_gdistances": True, "batch64_ms": t_batch,
                              "single_source_ms": ms.value / max(1, len(ss))}), flush=True)
        return

    bc_dev = ctypes.c_void_p()
    _lib.check(lib.lgbc_device_alloc(ctypes.byref(bc_dev), 8 * n))
    srcp = _lib.ptr(src)

    def step_dev():
        _lib.check(lib.lgbc_betweenness_dev(h, srcp, len(src), 0, bc_dev))

    for _ in range(args.warmup):
        step_dev()
    _lib.check(lib.lgbc_graph_sync(h))
    stats = dg.stats()

    clocks = Clocks(smi_index)
    dist.barrier()
    _lib.check(lib.lgbc_graph_sync(h))
    clocks.start()
    _lib.check(lib.lgbc_timer_start(h))
    for _ in range(args.steps):
        step_dev()
    ms = ctypes.c_double()
    launches = ctypes.c_int64()
    _lib.check(lib.lgbc_timer_stop(h, ctypes.byref(ms), ctypes.byref(launches)))
    clk = clocks.stop()
    dist.barrier()
    t_dev = dist.max(ms.value / 1e3)
    te_step = k_act * m
    value = dist.sum(te_step * args.steps) / t_dev / 1e9

    if args.profile_only:
        if dist.rank == 0:
            print(json.dumps({"profile_only": True, "ms_per_step": ms.value / args.steps,
                              "gpu_launches": int(launches.value)}), flush=True)
        lib.lgbc_device_free(bc_dev)
        return

    # bc result sanity: finite and non-negative
    host_bc = np.empty(n, np.float64)
    _lib.check(lib.lgbc_memcpy(_lib.ptr(host_bc), bc_dev, 8 * n, 2))
    assert np.all(np.isfinite(host_bc)) and host_bc.min() >= 0

    # ---- end to end through the C ABI with host buffers ----------------------------
    def pinned(a):
        p = ctypes.c_void_p()
        _lib.check(lib.lgbc_host_alloc(ctypes.byref(p), max(a.nbytes, 1)))
        ctypes.memmove(p, a.ctypes.data, a.nbytes)
        return p

    prp, pci = pinned(rp), pinned(ci)
    pirp = pici = None
    if directed:
        pirp, pici = pinned(irp), pinned(ici)
    out = np.empty(n, np.float64)

    def step_e2e():
        hh = ctypes.c_void_p()
        _lib.check(lib.lgbc_graph_create(ctypes.byref(hh), n, nnz, prp, pci, pirp, pici,
                                         int(directed)))
        try:
            t = _lib.LgbcTuning()
            for k_, _ in _lib.LgbcTuning._fields_:
                if k_ in tuning:
                    setattr(t, k_, tuning[k_])
            _lib.check(lib.lgbc_set_tuning(hh, ctypes.byref(t)))
            _lib.check(lib.lgbc_betweenness(hh, srcp, len(src), 0, _lib.ptr(out)))
        finally:
            lib.lgbc_graph_destroy(hh)

    e2e_steps = max(1, min(args.steps, 5))
    step_e2e()
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        step_e2e()
    t_e2e = dist.max((time.perf_counter() - t0) / e2e_steps)
    e2e_value = dist.sum(te_step) / t_e2e / 1e9
    for p_ in (prp, pci, pirp, pici):
        if p_ is not None:
            lib.lgbc_host_free(p_)

    # ---- gdistances from 64 sources (the workload's BFS part) ----------------------
    rng = np.random.default_rng(3 + dist.rank)
    gsrc = rng.choice(n, 64, replace=False).astype(np.int32)
    dist_out = np.empty((64, n), np.int32)
    _lib.check(lib.lgbc_gdistances_batch(h, _lib.ptr(gsrc), 64, _lib.ptr(dist_out)))
    _lib.check(lib.lgbc_timer_start(h))
    gd_reps = 3
    for _ in range(gd_reps):
        _lib.check(lib.lgbc_gdistances_batch(h, _lib.ptr(gsrc), 64, _lib.ptr(dist_out)))
    _lib.check(lib.lgbc_timer_stop(h, ctypes.byref(ms), None))
    gd_t = ms.value / 1e3 / gd_reps
    gd_active = int(np.count_nonzero(np.diff(rp)[gsrc] > 0))
    # single-source gdistances (the direction-optimising BFS of bfs.cu), 8 of
    # the sources one call each; each call's time includes its n-entry read-back
    one = np.empty(n, np.int32)
    ss = [np.array([s_], np.int32) for s_ in gsrc[np.diff(rp)[gsrc] > 0][:8]]
    for a in ss[:1]:
        _lib.check(lib.lgbc_gdistances(h, _lib.ptr(a), 1, _lib.ptr(one)))
    _lib.check(lib.lgbc_timer_start(h))
    for a in ss:
        _lib.check(lib.lgbc_gdistances(h, _lib.ptr(a), 1, _lib.ptr(one)))
    _lib.check(lib.lgbc_timer_stop(h, ctypes.byref(ms), None))
    ss_t = ms.value / 1e3 / max(1, len(ss))

    # ---- the double-float dependency variant (opt-in, narrower than FP64) ------------
    df32 = None
    if not tuning.get("dependency_df32", 0):
        dg.set_tuning(dependency_df32=1)
        try:
            step_dev()
            _lib.check(lib.lgbc_timer_start(h))
            df_steps = max(1, min(args.steps, 3))
            for _ in range(df_steps):
                step_dev()
            _lib.check(lib.lgbc_timer_stop(h, ctypes.byref(ms), None))
        finally:
            dg.set_tuning(dependency_df32=0)
        df_t = ms.value / 1e3 / df_steps
        df32 = {"value": te_step / df_t / 1e9, "unit": UNIT, "ms_per_step": df_t * 1e3,
                "dtype": dep_dtype({"dependency_df32": 1}),
                "note": "opt-in variant (tuning dependency_df32=1); not the headline"}

    # ---- roofline --------------------------------------------------------------------
    peak, peak_kind = peak_hbm()
    t_step = t_dev / args.steps
    abytes = bc_algorithmic_bytes(n, nnz, k_act, max(1, min(128, int(tuning["lanes"]))))
    achieved = abytes / t_step / 1e9
    # the committed capture is of the default workload (R-MAT 20, k = 4096) only
    traffic = (traffic_per_step() if args.workload == "c2" and args.scale == 20
               and len(src) == 4096 else None)

    # ---- CPU baseline (rank 0, N = 1 only) -------------------------------------------
    cpu = None
    gd_cpu = None
    if dist.world == 1 and not args.no_cpu:
        nthreads = os.cpu_count() or 1
        cpu_v, cpu_t, cpu_n = cpu_betweenness_sample(g, src, nthreads, args.cpu_seconds, 7)
        cpu = {"value": cpu_v, "unit": UNIT, "cores": nthreads, "kind": "port",
               "sample": f"{cpu_n} of the {k_act} active sources ({cpu_t:.1f} s), faithful "
                         "heap-Dijkstra restatement of src/shortestpaths/dijkstra.jl:59-141 + "
                         "_accumulate_basic!, one source per thread"}
        fv, ft, fn = cpu_betweenness_sample(g, src, nthreads, args.cpu_seconds / 3, 8,
                                            mode="fast")
        cpu["fast_mode"] = {"value": fv, "unit": UNIT, "cores": nthreads, "kind": "port",
                            "sample": f"{fn} of the {k_act} active sources ({ft:.1f} s), BFS "
                                      "Brandes with the same values, one source per thread"}
        from oracle import oracle
        oracle.gdistances_many(rp, ci, gsrc[:nthreads], nthreads=nthreads)
        t0 = time.perf_counter()
        oracle.gdistances_many(rp, ci, gsrc, nthreads=nthreads)
        gcpu_t = time.perf_counter() - t0
        gd_cpu = {"ms": gcpu_t * 1e3, "gteps": gd_active * m / gcpu_t / 1e9, "cores": nthreads,
                  "kind": "port",
                  "sample": "the same 64 sources: the gdistances! restatement "
                            "(src/traversals/bfs.jl:95-124), one source per thread"}

    if dist.rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": dep_dtype(tuning), "data": "synthetic",
            "config": {"workload": wname, "description": WORKLOADS[args.workload],
                       "n": n, "m": m, "nnz": nnz, "directed": directed, "sources": len(src),
                       "active_sources": k_act, "lanes": tuning["lanes"], "tuning": tuning,
                       "autotune_s": tune_s,
                       "parallelism": f"replicas x{dist.world}",
                       "l2": ("inputs larger than L2 (CSR + lane state); no flush"
                              if nnz * 4 + n * 1024 > 129e6 else
                              "small graph: inputs fit in L2, no flush (parity config)")},
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": (8 * (n + 1) + 4 * nnz) * (2 if directed else 1)
                    + 4 * len(src),
                    "d2h_bytes_per_step": 8 * n,
                    "ms_per_step": t_e2e * 1e3},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "peak_source": f"{peak_kind} hbm_gbs",
                         "algorithmic_bytes_per_step": abytes,
                         "scope": "whole Brandes pass (all kernels of one step)"},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": int(launches.value),
            "kernel_stats_per_step": stats,
            "gdistances": {"sources": 64, "active": gd_active, "ms": gd_t * 1e3,
                           "gteps": gd_active * m / gd_t / 1e9,
                           "algorithmic_gbs": gd_algorithmic_bytes(n, nnz, 64) / gd_t / 1e9,
                           "roofline_frac": gd_algorithmic_bytes(n, nnz, 64) / gd_t / 1e9 / peak,
                           "cpu": gd_cpu,
                           "single_source": {
                               "sources": len(ss), "ms_per_call": ss_t * 1e3,
                               "gteps": m / ss_t / 1e9,
                               "algorithmic_gbs": gd_algorithmic_bytes(n, nnz, 1) / ss_t / 1e9,
                               "note": "one lgbc_gdistances call per source, its 4n-byte "
                                       "result read back inside the timed region"}},
            "df32_variant": df32,
        }
        print(json.dumps(line), flush=True)
    lib.lgbc_device_free(bc_dev)


def run_ours_many(args, dist: Dist):
    """Config C3: exact BC of many BA graphs in one lgbc_betweenness_many call
    per step (host buffers in, raw vectors out)."""
    import lgbc
    graphs = many_graphs(dist.rank, args.graphs)
    te = sum(g.nv() * g.ne() for g in graphs)  # every vertex is an active source
    log(f"[rank {dist.rank}] {len(graphs)} BA graphs, sum n = {sum(g.nv() for g in graphs)}, "
        f"traversed edges per step = {te:.3g}")
    for _ in range(args.warmup):
        lgbc.betweenness_centrality_many(graphs, normalize=False)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        lgbc.betweenness_centrality_many(graphs, normalize=False)
    t = dist.max((time.perf_counter() - t0) / args.steps)
    value = dist.sum(te) / t / 1e9
    if dist.rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u64 path counts, f64 dependencies", "data": "synthetic",
            "config": {"workload": f"ba_many_{len(graphs)}_exact_bc", "description": WORKLOADS["c3"],
                       "graphs": len(graphs), "graphs_per_s": len(graphs) / t},
            "e2e": {"value": value, "unit": UNIT,
                    "h2d_bytes_per_step": sum(8 * (g.nv() + 1) + 4 * 2 * g.ne() for g in graphs),
                    "d2h_bytes_per_step": 8 * sum(g.nv() for g in graphs)},
        }), flush=True)


def run_reference_many(args, nthreads: int):
    """C3 on the host cores: the faithful oracle on a bounded sample of graphs."""
    from oracle import oracle
    graphs = many_graphs(0, args.graphs, gen=oracle)
    rng = np.random.default_rng(5)
    per_step = []
    for it in range(args.warmup + args.steps):
        idx = rng.choice(len(graphs), 2, replace=False)
        te = 0
        t = time.perf_counter()
        for i in idx:
            g = graphs[i]
            rp, ci = g.csr()
            srcs = np.arange(min(g.nv(), 16 * nthreads), dtype=np.int32)
            oracle.betweenness_raw(rp, ci, srcs, mode="faithful", nthreads=nthreads)
            te += len(srcs) * g.ne()
        dt = time.perf_counter() - t
        if it >= args.warmup:
            per_step.append((te, dt))
    te = sum(a for a, _ in per_step)
    dt = sum(b for _, b in per_step)
    value = te / dt / 1e9
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": f"ba_many_{len(graphs)}_exact_bc"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": "2 graphs per step, 16 sources per thread each"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def run_c5_kernels(args):
    """The learned proposal's kernels on one graph (for profiling): core
    numbers and features, the MLP forward over every vertex with the softmax
    CDF, and one training gradient over 65,536 rows; GPU times by CUDA events."""
    import lgbc
    from lgbc import compare
    from lgbc import generators as G
    g = G.rmat(args.scale, 16, seed=1)
    with compare._Timer(g) as tf:
        f = lgbc.features(g)
    passes = g.device_handle().stats()["levels"]
    m = lgbc.SourceProposal(seed=0)
    m.set_norm(f.mean(0), np.maximum(f.std(0), 1e-6))
    with compare._Timer(g) as tb:
        m.build(g, 0.1)
    rows = min(65536, g.nv())
    x = f[:rows]
    t = np.log1p(np.arange(rows, dtype=np.float32) % 97)
    t0 = time.perf_counter()
    m.grad(x, t)
    grad_s = time.perf_counter() - t0
    print(json.dumps({"c5_kernels": {"n": g.nv(), "m": g.ne(), "features_ms": tf.ms,
                                     "core_passes": passes, "proposal_build_ms": tb.ms,
                                     "grad_rows": rows, "grad_call_ms": grad_s * 1e3}}), flush=True)
    m.close()


CEILING_ARMS = ("mass", "sqrt_mass", "uniform_active")


def ceiling_arms(compare, g, exact_bc, ks, args, recs):
    """Adds the fixed-proposal arms built from exact per-source masses (what a
    perfect predictor of the network's target could reach) to ``recs``."""
    methods = ("learned", "learned_systematic")
    if not args.c5_ceiling:
        return recs, methods, None
    props, mass_ms = compare.ceiling_proposals(g)
    arms = tuple(name for name in CEILING_ARMS if name in props)
    for name in arms:
        recs = recs + compare.run_fixed(g, exact_bc, props[name], ks, name, seeds=args.c5_seeds)
    return recs, methods + arms, mass_ms


def run_c5(args, dist: Dist):
    """Config C5: train the proposal on 128 R-MAT scale-14 + 128 BA graphs,
    then compare uniform and learned sampling against exact BC on (a) the
    R-MAT scale-20 graph and (b) the induced subgraph of a 10^5-vertex BFS
    ball of R-MAT scale 24 (plus the proposal build and one sampled BC on the
    whole scale-24 graph, time only)."""
    import lgbc
    from lgbc import compare
    from lgbc import generators as G
    if dist.rank != 0:
        return
    out = {}
    t = time.perf_counter()
    train = compare.training_graphs(args.c5_train, args.c5_train, args.c5_train_scale)
    prop, info = compare.train_default(train, steps=args.c5_steps)
    info["generate_s"] = time.perf_counter() - t - info["fit_s"]
    out["training"] = info
    log(f"trained: {info}")
    kt = [1024, 4096, 16384]
    ks_u = [1024, 2048, 4096, 8192, 16384]
    ks_l = [256, 512, 1024, 2048, 4096, 8192, 16384]
    evals = {}
    # (a) R-MAT scale 20, the same graph as the sampled-BC workload
    g = G.rmat(args.scale, 16, seed=1)
    ex, ex_ms = compare.exact(g)
    st = g.device_handle().stats()
    log(f"exact BC on rmat{args.scale}: {ex_ms / 1e3:.1f} s, {st['active_sources']} active sources")
    recs, build_ms = compare.run_estimators(g, ex, prop, ks_u, ks_l, seeds=args.c5_seeds)
    recs, methods, mass_ms = ceiling_arms(compare, g, ex, ks_l, args, recs)
    evals[f"rmat{args.scale}"] = dict(n=g.nv(), m=g.ne(), exact_ms=ex_ms, mass_ms=mass_ms,
                                      **compare.summarise(recs, build_ms, kt, methods))
    log(json.dumps(evals[f"rmat{args.scale}"]["equal_error"]))
    g.device_handle().close()
    del g
    # (b) BFS ball of R-MAT scale 24 around a random non-isolated vertex
    if args.c5_ball_scale > 0:
        t = time.perf_counter()
        big = G.rmat(args.c5_ball_scale, 16, seed=1)
        gen_s = time.perf_counter() - t
        deg = big.degrees()
        rng = np.random.default_rng(24)
        cand = np.flatnonzero(deg > 0)
        center = int(cand[rng.integers(len(cand))])
        # proposal build and one sampled BC per method on the whole graph (time only)
        with compare._Timer(big) as tb:
            prop.build(big, 0.1)
        src = np.asarray(lgbc.sample(big.vertices(), 1024, rng=np.random.default_rng(3)))
        with compare._Timer(big) as tu:
            lgbc.betweenness_centrality(big, src)
        k_act_u = big.device_handle().stats()["active_sources"]
        with compare._Timer(big) as tl:
            lgbc.betweenness_centrality_learned(big, 1024, prop, seed=3, build=False)
        k_act_l = big.device_handle().stats()["active_sources"]
        whole = dict(n=big.nv(), m=big.ne(), generate_s=gen_s, proposal_build_ms=tb.ms,
                     uniform_k1024_ms=tu.ms, uniform_active=k_act_u,
                     uniform_gteps=k_act_u * big.ne() / (tu.ms * 1e-3) / 1e9,
                     learned_k1024_ms=tl.ms, learned_active=k_act_l,
                     learned_gteps=k_act_l * big.ne() / (tl.ms * 1e-3) / 1e9)
        log(f"rmat{args.c5_ball_scale}: {whole}")
        sub, _ = compare.bfs_ball(big, center, args.c5_ball)
        big.device_handle().close()
        del big
        ex, ex_ms = compare.exact(sub)
        recs, build_ms = compare.run_estimators(sub, ex, prop, ks_u, ks_l, seeds=args.c5_seeds)
        recs, methods, mass_ms = ceiling_arms(compare, sub, ex, ks_l, args, recs)
        evals[f"rmat{args.c5_ball_scale}_ball{args.c5_ball}"] = dict(
            n=sub.nv(), m=sub.ne(), center=center, exact_ms=ex_ms, mass_ms=mass_ms,
            whole_graph=whole, **compare.summarise(recs, build_ms, kt, methods))
        log(json.dumps(evals[f"rmat{args.c5_ball_scale}_ball{args.c5_ball}"]["equal_error"]))
    out["evaluations"] = evals
    # time ratio at equal L1 per graph and budget, learned (with build) and the ceiling arms
    ceiling = {}
    for name, e in evals.items():
        per_k = {}
        for r in e["equal_error"]:
            row = {"learned": r["time_ratio_with_build"]}
            for m in CEILING_ARMS:
                for x in e.get("equal_error_" + m, []):
                    if x["k_uniform"] == r["k_uniform"]:
                        row[m] = x["time_ratio"]
            per_k[str(r["k_uniform"])] = row
        ceiling[name] = per_k
    out["ceiling"] = ceiling
    log(json.dumps(out["ceiling"]))
    main_eval = evals[f"rmat{args.scale}"]
    head = next(r for r in main_eval["equal_error"] if r["k_uniform"] == 4096)
    head_sys = next(r for r in main_eval["equal_error_systematic"] if r["k_uniform"] == 4096)
    print(json.dumps({
        "metric": "GPU time of learned sampling at uniform sampling's L1 error, relative to uniform",
        "value": head["time_ratio_with_build"], "unit": "ratio", "n_gpus": 1,
        "steps": sum(len(e["uniform"]) + len(e["learned"]) + len(e["learned_systematic"])
                     + sum(len(e.get(m, [])) for m in CEILING_ARMS)
                     for e in evals.values()) * args.c5_seeds,
        "warmup": 0, "ms_per_step": None, "higher_is_better": False, "scaling": "none",
        "vs_baseline": None, "dtype": "u64 path counts, f64 weighted dependencies; MLP bf16/f32",
        "data": "synthetic",
        "config": {"workload": f"learned_vs_uniform_rmat{args.scale}_k4096",
                   "description": WORKLOADS["c5"], "seeds": args.c5_seeds,
                   "proposal_eps": 0.1, "sampling": "iid (value); systematic in c5",
                   "systematic_time_ratio_with_build": head_sys["time_ratio_with_build"]},
        "c5": out,
    }), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="c2",
                    help="; ".join(f"{k}: {v}" for k, v in WORKLOADS.items()))
    ap.add_argument("--scale", type=int, default=20)
    ap.add_argument("--k", type=int, default=0, help="sampled sources (0 = the workload's)")
    ap.add_argument("--graphs", type=int, default=4096, help="c3: number of graphs")
    ap.add_argument("--tuning", default="", help="lgbc_tuning overrides, e.g. source_order=0,hub_degree=512")
    ap.add_argument("--autotune", action="store_true", help="run lgbc_tune before timing")
    ap.add_argument("--c5-train", type=int, default=128, help="c5: training graphs per family")
    ap.add_argument("--c5-train-scale", type=int, default=14)
    ap.add_argument("--c5-steps", type=int, default=3000, help="c5: training steps")
    ap.add_argument("--c5-seeds", type=int, default=8)
    ap.add_argument("--c5-ball-scale", type=int, default=24, help="c5: 0 skips the ball graph")
    ap.add_argument("--c5-ball", type=int, default=100000)
    ap.add_argument("--c5-ceiling", type=int, default=1,
                    help="c5: 1 adds the proposals built from exact masses (0 skips them)")
    ap.add_argument("--c5-kernels", action="store_true",
                    help="c5: only run the proposal's kernels once on R-MAT --scale (profiling)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0,
                    help="approximate CPU-baseline sample length")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--profile-only", action="store_true",
                    help="run only the device-resident steps (for ncu launch lists)")
    ap.add_argument("--profile-gdistances", action="store_true",
                    help="run only the workload's gdistances calls (for ncu launch lists)")
    ap.add_argument("--profile-batch", type=int, default=None,
                    help="run only batch B (128 sources, in the library's source order) of the "
                         "workload: a one-batch case of the full step for profiling")
    args = ap.parse_args()
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        elif args.workload == "c5" and args.c5_kernels:
            run_c5_kernels(args)
        elif args.workload == "c5":
            run_c5(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
