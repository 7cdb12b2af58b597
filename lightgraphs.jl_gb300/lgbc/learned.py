"""Learned source proposal for sampled betweenness centrality.

LightGraphs' k-sampled ``betweenness_centrality(g, k)`` draws k distinct
sources uniformly (src/centrality/betweenness.jl:77-78, src/utils.jl:12-45)
and rescales by n/k.  This module adds an importance-sampled estimator next to
it (it has no counterpart in the reference):

    raw(v) = sum_i delta_{s_i}(v) / (k p_{s_i}),   s_i drawn i.i.d. from p,

which is unbiased for the exact raw betweenness; ``_rescale!(raw, n,
normalize, directed, n)`` then gives the scale of the exact call (uniform
p = 1/n reproduces the n/k factor).  The proposal is

    p = (1 - eps) softmax(MLP(features)) + eps / n,    eps = 0.1 by default,

a defensive mixture (Hesterberg 1995) that keeps every weight below
n / (eps k).  The MLP (4 -> 64 -> 64 -> 1, BF16 weights, FP32 accumulation,
trained on the GPU by the library's own forward / backward kernels) predicts
log(1 + dependency mass) of a source, sum_v delta_s(v), from four structural
features: log(1 + degree), log(1 + core number) (core_number,
src/degeneracy.jl:38-80), the mean log(1 + degree) of the neighbours and
log(1 + the neighbours' degree sum).  Training targets are exact masses from
the GPU's multi-source BFS.  Uniform sampling (``betweenness_centrality(g,
k)``) and the exact call stay available as the fallback and as the yardstick
of the estimator's error.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _lib
from .centrality import _rescale_, _sources0


def _need_undirected(g, what: str) -> None:
    if g.is_directed():
        raise _lib.MethodError(f"{what} covers undirected graphs")


def core_number(g) -> np.ndarray:
    """core_number(g) (src/degeneracy.jl:38-96) on the GPU: int32 vector
    indexed by vertex - 1 (digraphs: arcs count at both ends).  Raises
    ArgumentError for a graph with self-loops, as the reference does."""
    out = np.empty(g.nv(), np.int32)
    if g.nv() == 0:
        return out
    _lib.check(_lib.lib().lgbc_core_number(g.device_handle().handle, _lib.ptr(out)))
    return out


def features(g) -> np.ndarray:
    """The proposal's per-vertex features, float32 array of shape (n, 4)."""
    _need_undirected(g, "features")
    out = np.empty((g.nv(), 4), np.float32)
    if g.nv() == 0:
        return out
    _lib.check(_lib.lib().lgbc_features(g.device_handle().handle, _lib.ptr(out)))
    return out


def dependency_mass(g, vs=None) -> np.ndarray:
    """sum_{v != s} delta_s(v) for each source s in ``vs`` (1-based; default
    all vertices), exact: sum over reached t != s of (d(s, t) - 1)."""
    src = np.arange(g.nv(), dtype=np.int32) if vs is None else _sources0(g, vs)
    out = np.empty(len(src), np.float64)
    if len(src) == 0:
        return out
    src = np.ascontiguousarray(src, np.int32)
    _lib.check(_lib.lib().lgbc_dependency_mass(g.device_handle().handle, _lib.ptr(src), len(src),
                                               _lib.ptr(out)))
    return out


def betweenness_raw_weighted(g, src0: np.ndarray, w: np.ndarray) -> np.ndarray:
    """Unscaled sum_i w[i] delta_{src0[i]}(v) over 0-based sources (repeats allowed)."""
    src = np.ascontiguousarray(src0, np.int32)
    ww = np.ascontiguousarray(w, np.float64)
    if src.shape != ww.shape:
        raise _lib.ArgumentError("sources and weights differ in length")
    out = np.empty(g.nv(), np.float64)
    if g.nv() == 0:
        return out
    _lib.check(_lib.lib().lgbc_betweenness_weighted(g.device_handle().handle, _lib.ptr(src),
                                                    _lib.ptr(ww), len(src), _lib.ptr(out)))
    return out


class SourceProposal:
    """The proposal network (an ``lgbc_mlp`` handle on the current GPU)."""

    PARAMS = _lib.MLP_PARAMS

    def __init__(self, seed: int = 0):
        self._h = ctypes.c_void_p()
        _lib.check(_lib.lib().lgbc_mlp_create(ctypes.byref(self._h), int(seed) & (2**64 - 1)))

    # -- lifetime -----------------------------------------------------------
    def close(self) -> None:
        if self._h:
            _lib.lib().lgbc_mlp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- parameters ---------------------------------------------------------
    def params(self) -> np.ndarray:
        out = np.empty(self.PARAMS, np.float32)
        _lib.check(_lib.lib().lgbc_mlp_get_params(self._h, _lib.ptr(out), None))
        return out

    def params_bf16(self) -> np.ndarray:
        """The BF16 working copy, widened exactly to float32."""
        bits = np.empty(self.PARAMS, np.uint16)
        _lib.check(_lib.lib().lgbc_mlp_get_params(self._h, None, _lib.ptr(bits)))
        return (bits.astype(np.uint32) << 16).view(np.float32)

    def set_params(self, p) -> None:
        a = np.ascontiguousarray(p, np.float32)
        if a.shape != (self.PARAMS,):
            raise _lib.ArgumentError(f"expected {self.PARAMS} parameters")
        _lib.check(_lib.lib().lgbc_mlp_set_params(self._h, _lib.ptr(a)))

    def norm(self):
        mu = np.empty(4, np.float32)
        sd = np.empty(4, np.float32)
        _lib.check(_lib.lib().lgbc_mlp_get_norm(self._h, _lib.ptr(mu), _lib.ptr(sd)))
        return mu, sd

    def set_norm(self, mean, stdev) -> None:
        mu = np.ascontiguousarray(mean, np.float32)
        sd = np.ascontiguousarray(stdev, np.float32)
        _lib.check(_lib.lib().lgbc_mlp_set_norm(self._h, _lib.ptr(mu), _lib.ptr(sd)))

    def save(self, path: str) -> None:
        mu, sd = self.norm()
        np.savez(path, params=self.params(), mean=mu, stdev=sd)

    @classmethod
    def load(cls, path: str) -> "SourceProposal":
        z = np.load(path)
        m = cls()
        m.set_params(z["params"])
        m.set_norm(z["mean"], z["stdev"])
        return m

    # -- network --------------------------------------------------------------
    def forward(self, x) -> np.ndarray:
        a = np.ascontiguousarray(x, np.float32).reshape(-1, 4)
        y = np.empty(a.shape[0], np.float32)
        _lib.check(_lib.lib().lgbc_mlp_forward(self._h, _lib.ptr(a), a.shape[0], _lib.ptr(y)))
        return y

    def grad(self, x, target):
        """(gradient, loss) of the centred squared error over one batch."""
        a = np.ascontiguousarray(x, np.float32).reshape(-1, 4)
        t = np.ascontiguousarray(target, np.float32).ravel()
        g = np.empty(self.PARAMS, np.float32)
        loss = ctypes.c_float()
        _lib.check(_lib.lib().lgbc_mlp_grad(self._h, _lib.ptr(a), _lib.ptr(t), a.shape[0],
                                            _lib.ptr(g), ctypes.byref(loss)))
        return g, float(loss.value)

    def train(self, x, target, group_off, *, steps=3000, batch=1024, warmup=100, lr=3e-3,
              lr_final=3e-4, beta1=0.9, beta2=0.999, eps=1e-8, seed=0) -> np.ndarray:
        """Adam on the GPU over grouped rows; returns the per-step losses."""
        a = np.ascontiguousarray(x, np.float32).reshape(-1, 4)
        t = np.ascontiguousarray(target, np.float32).ravel()
        off = np.ascontiguousarray(group_off, np.int64)
        cfg = _lib.LgbcTrainCfg(int(steps), int(batch), int(warmup), float(lr), float(lr_final),
                                float(beta1), float(beta2), float(eps), int(seed) & (2**64 - 1))
        losses = np.empty(max(int(steps), 1), np.float32)
        _lib.check(_lib.lib().lgbc_mlp_train(self._h, _lib.ptr(a), _lib.ptr(t), a.shape[0],
                                             _lib.ptr(off), len(off) - 1, ctypes.byref(cfg),
                                             _lib.ptr(losses)))
        return losses[:int(steps)]

    def fit(self, graphs, *, sources_per_graph: int = 1024, seed: int = 0, **train_kw) -> dict:
        """Train on generated graphs: features of a uniform sample of each
        graph's vertices, targets log(1 + exact dependency mass)."""
        rng = np.random.default_rng(seed)
        xs, ts, off = [], [], [0]
        for g in graphs:
            n = g.nv()
            m = min(int(sources_per_graph), n)
            src = np.sort(rng.choice(n, size=m, replace=False)).astype(np.int32)
            f = features(g)[src]
            mass = dependency_mass(g, src + 1)
            xs.append(f)
            ts.append(np.log1p(mass).astype(np.float32))
            off.append(off[-1] + m)
        x = np.concatenate(xs)
        t = np.concatenate(ts)
        mu = x.mean(axis=0)
        sd = x.std(axis=0)
        sd = np.where(sd > 1e-6, sd, 1.0)
        self.set_norm(mu, sd)
        losses = self.train(x, t, np.array(off, np.int64), seed=seed, **train_kw)
        return {"rows": int(len(t)), "graphs": len(off) - 1, "losses": losses}

    # -- proposal on a graph ------------------------------------------------
    def build(self, g, eps: float = 0.1, return_p: bool = False):
        """Features, scores, p and its CDF for g on the device (kept in g's handle)."""
        _need_undirected(g, "the learned proposal")
        p = np.empty(g.nv(), np.float64) if return_p else None
        _lib.check(_lib.lib().lgbc_proposal_build(g.device_handle().handle, self._h, float(eps),
                                                  _lib.ptr(p)))
        return p

    @staticmethod
    def sample(g, k: int, seed: int = 0, scheme: str = "iid"):
        """k 0-based sources from g's built proposal and their weights 1/(k p):
        ``scheme`` "iid" (independent draws) or "systematic" (one random
        offset, draw i at (i + U)/k of the CDF; unbiased, lower variance)."""
        code = {"iid": _lib.SAMPLE_IID, "systematic": _lib.SAMPLE_SYSTEMATIC}.get(scheme)
        if code is None:
            raise _lib.ArgumentError(f"unknown sampling scheme {scheme!r}")
        src = np.empty(int(k), np.int32)
        w = np.empty(int(k), np.float64)
        _lib.check(_lib.lib().lgbc_proposal_sample(g.device_handle().handle, int(k),
                                                   int(seed) & (2**64 - 1), code, _lib.ptr(src),
                                                   _lib.ptr(w)))
        return src, w


def betweenness_centrality_learned(g, k: int, proposal: SourceProposal, *, normalize: bool = True,
                                   eps: float = 0.1, seed: int = 0, build: bool = True,
                                   scheme: str = "iid", timings: dict | None = None) -> np.ndarray:
    """Importance-sampled betweenness with k sources drawn from the learned
    proposal (``scheme`` "iid" or "systematic"), scaled like
    betweenness_centrality(g; normalize).  With ``build=False`` the proposal
    already built for g is reused.  ``timings`` (a dict) receives wall-clock
    seconds of the build and sampled parts."""
    n = g.nv()
    t0 = time.perf_counter()
    if build:
        proposal.build(g, eps)
    t1 = time.perf_counter()
    src, w = proposal.sample(g, k, seed, scheme)
    raw = betweenness_raw_weighted(g, src, w)
    _rescale_(raw, n, normalize, g.is_directed(), n)
    t2 = time.perf_counter()
    if timings is not None:
        timings["build_s"] = t1 - t0
        timings["sample_bc_s"] = t2 - t1
    return raw


def l1_error(est: np.ndarray, exact: np.ndarray) -> float:
    """||est - exact||_1 / ||exact||_1."""
    den = float(np.abs(exact).sum())
    return float(np.abs(est - exact).sum()) / den if den > 0 else float(np.abs(est).sum())


def top_rank_error(est: np.ndarray, exact: np.ndarray, frac: float = 0.01) -> float:
    """1 - |top(est) & top(exact)| / ceil(frac n), ties broken by vertex id."""
    n = len(exact)
    m = int(np.ceil(frac * n))
    if m == 0:
        return 0.0
    a = set(np.lexsort((np.arange(n), -est))[:m].tolist())
    b = set(np.lexsort((np.arange(n), -exact))[:m].tolist())
    return 1.0 - len(a & b) / m
