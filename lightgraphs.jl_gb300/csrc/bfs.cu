// bfs.cu -- direction-optimising level-synchronous BFS for gdistances.
//
// Replaces gdistances! (src/traversals/bfs.jl:95-124) and its threaded
// variant (src/Parallel/traversals/gdistances.jl:36-116): every source gets
// level 0, every other vertex the level at which the BFS first reaches it,
// INT32_MAX where nothing reaches it.  The per-level sort of the reference
// (bfs.jl:121) only fixes visiting order and does not change any distance.
//
// Top-down levels expand the frontier queue over out-edges with degree-binned
// thread mapping: a warp takes 32 frontier vertices and streams their
// concatenated out-lists 32 edges at a time, so a lane never idles on a short
// list; a vertex with more than kBfsLarge out-edges (an R-MAT hub has 65K) is
// deferred to a list whose edges the whole grid expands in a second kernel.
// atomicCAS on the distance claims a vertex once.
// Bottom-up levels give each unvisited vertex one thread that scans its
// in-edges and stops at the first in-neighbour in the frontier bitmap; the
// bitmap is staged in shared memory when it fits, and a warp owns 32
// consecutive vertices, so it writes one bitmap word of the next frontier
// (its ballot) without atomics and appends its discoveries with one atomic.
#include <algorithm>

#include "lgbc_kernels.h"

namespace lgbc {
namespace {

__device__ __forceinline__ long long gwarp() {
  return (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
}
__device__ __forceinline__ long long nwarps() {
  return (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
}

__device__ __forceinline__ int64_t shfl_i64(int64_t x, int src) {
  return static_cast<int64_t>(shfl_u64(static_cast<uint64_t>(x), src));
}

__device__ __forceinline__ uint32_t* bm_at(const BfsBuffers& b, int level) {
  return (level & 1) ? b.bm[1] : b.bm[0];
}

__global__ void k_bfs_ctl_reset(BatchCtl* c) {
  c->lo = 0;
  c->hi = 0;
  c->tail = 0;
  c->mf = 0;
  c->mf_cur = 0;
  c->mu_done = 0;
  c->cap = 0;
  c->level = 0;
  c->maxlevel = 0;
  c->done = 0;
  c->overflow_list = 0;
  c->overflow_sigma = 0;
  c->mode = 0;
  c->large = 0;
}

// Level 0: claim each source once (duplicates in the source list are
// harmless, as in bfs.jl:103-107).
__global__ void k_bfs_seed(DevGraph g, BfsBuffers b, const int32_t* src, int64_t nsrc,
                           int32_t* dist) {
  BatchCtl* c = b.ctl;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < nsrc;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int32_t s = src[i];
    if (atomicCAS(dist + s, kUnreached, 0) == kUnreached) {
      const unsigned long long slot = atomicAdd(&c->tail, 1ull);
      b.queue[slot] = s;
      atomicOr(&b.bm[0][s >> 5], 1u << (s & 31));
      atomicAdd(&c->mf, static_cast<unsigned long long>(g.rowptr[s + 1] - g.rowptr[s]));
      atomicAdd(&c->mu_done,
                static_cast<unsigned long long>(g.in_rowptr[s + 1] - g.in_rowptr[s]));
    }
  }
}

__global__ void k_bfs_seed_done(BatchCtl* c) {
  c->lo = 0;
  c->hi = c->tail;
  c->mf_cur = c->mf;
  c->mf = 0;
  if (c->tail == 0) {
    c->done = 1;
    c->maxlevel = -1;
  }
}

// Zero the bitmap that the coming top-down level fills with atomicOr, and the
// level's deferred-vertex count.
__global__ void k_bfs_clear_next(BfsBuffers b, int64_t nwords) {
  uint32_t* nbm = bm_at(b, b.ctl->level + 1);
  if (blockIdx.x == 0 && threadIdx.x == 0) b.ctl->large = 0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < nwords;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    nbm[i] = 0u;
}

// Claim w for level nl if no one has; returns whether this thread did.
__device__ __forceinline__ bool bfs_claim(const DevGraph& g, uint32_t* nbm, int32_t* dist,
                                          int32_t w, int32_t nl, unsigned long long& mf,
                                          unsigned long long& mu) {
  if (dist[w] != kUnreached || atomicCAS(dist + w, kUnreached, nl) != kUnreached) return false;
  atomicOr(nbm + (w >> 5), 1u << (w & 31));
  mf += static_cast<unsigned long long>(g.rowptr[w + 1] - g.rowptr[w]);
  mu += static_cast<unsigned long long>(g.in_rowptr[w + 1] - g.in_rowptr[w]);
  return true;
}

__device__ __forceinline__ void bfs_flush_counts(BatchCtl* c, unsigned long long mf,
                                                 unsigned long long mu) {
  mf = warp_sum_u64(mf);
  mu = warp_sum_u64(mu);
  if (lane_id() == 0) {
    if (mf) atomicAdd(&c->mf, mf);
    if (mu) atomicAdd(&c->mu_done, mu);
  }
}

// Top-down level: lane j of a warp holds frontier entry base + j.  Vertices
// with more than kBfsLarge out-edges go to b.large (when there is one); the
// others' out-lists are walked as one concatenation, edge k of it by lane
// k % 32 (the owning vertex found by a binary search over the warp's
// inclusive degree scan).
__global__ void __launch_bounds__(256) k_bfs_td(DevGraph g, BfsBuffers b, int32_t* dist) {
  BatchCtl* c = b.ctl;
  const unsigned long long lo = c->lo, hi = c->hi;
  const int32_t nl = c->level + 1;
  uint32_t* nbm = bm_at(b, nl);
  const int ln = lane_id();
  unsigned long long mf = 0, mu = 0;
  for (unsigned long long base = lo + static_cast<unsigned long long>(gwarp()) * kWarp; base < hi;
       base += static_cast<unsigned long long>(nwarps()) * kWarp) {
    const unsigned long long i = base + ln;
    int32_t v = 0;
    int64_t e0 = 0, deg = 0;
    if (i < hi) {
      v = b.queue[i];
      e0 = g.rowptr[v];
      deg = g.rowptr[v + 1] - e0;
    }
    const bool defer = b.large != nullptr && deg > kBfsLarge;
    const unsigned long long slot = warp_append(defer, &c->large);
    if (defer) b.large[slot] = v;
    const int d = defer ? 0 : static_cast<int>(deg);
    int incl = d;
#pragma unroll
    for (int o = 1; o < kWarp; o <<= 1) {
      const int y = __shfl_up_sync(kFull, incl, o);
      if (ln >= o) incl += y;
    }
    const int total = __shfl_sync(kFull, incl, kWarp - 1);
    const int off = incl - d;
    for (int k0 = 0; k0 < total; k0 += kWarp) {
      const int k = k0 + ln;
      int j = 0;  // the lane whose list holds concatenated edge k: the first with incl > k
#pragma unroll
      for (int step = 16; step >= 1; step >>= 1) {
        const int iv = __shfl_sync(kFull, incl, j + step - 1);
        if (iv <= k) j += step;
      }
      const int64_t ej = shfl_i64(e0, j);
      const int oj = __shfl_sync(kFull, off, j);
      bool app = false;
      int32_t w = 0;
      if (k < total) {
        w = g.colidx[ej + (k - oj)];
        app = bfs_claim(g, nbm, dist, w, nl, mf, mu);
      }
      const unsigned long long q = warp_append(app, &c->tail);
      if (app) b.queue[q] = w;
    }
  }
  bfs_flush_counts(c, mf, mu);
}

// The deferred high-degree frontier vertices: for each in turn, the whole
// grid walks its out-list (a warp takes 32 consecutive edges).
__global__ void __launch_bounds__(256) k_bfs_td_large(DevGraph g, BfsBuffers b, int32_t* dist) {
  BatchCtl* c = b.ctl;
  const unsigned long long nlarge = c->large;
  if (nlarge == 0) return;
  const int32_t nl = c->level + 1;
  uint32_t* nbm = bm_at(b, nl);
  const int ln = lane_id();
  unsigned long long mf = 0, mu = 0;
  for (unsigned long long h = 0; h < nlarge; ++h) {
    const int32_t v = b.large[h];
    const int64_t e0 = g.rowptr[v], e1 = g.rowptr[v + 1];
    for (int64_t e = e0 + gwarp() * kWarp; e < e1; e += nwarps() * kWarp) {
      const int64_t idx = e + ln;
      bool app = false;
      int32_t w = 0;
      if (idx < e1) {
        w = g.colidx[idx];
        app = bfs_claim(g, nbm, dist, w, nl, mf, mu);
      }
      const unsigned long long q = warp_append(app, &c->tail);
      if (app) b.queue[q] = w;
    }
  }
  bfs_flush_counts(c, mf, mu);
}

template <bool STAGE>
__global__ void __launch_bounds__(1024) k_bfs_bu(DevGraph g, BfsBuffers b, int32_t* dist) {
  extern __shared__ uint32_t sbm[];
  BatchCtl* c = b.ctl;
  const int32_t nl = c->level + 1;
  const int64_t n = g.n;
  const int64_t nwords = (n + 31) >> 5;
  const uint32_t* fbm = bm_at(b, nl - 1);
  uint32_t* nbm = bm_at(b, nl);
  if (STAGE) {
    const uint4* src4 = reinterpret_cast<const uint4*>(fbm);
    uint4* dst4 = reinterpret_cast<uint4*>(sbm);
    const int64_t n4 = nwords >> 2;
    for (int64_t i = threadIdx.x; i < n4; i += blockDim.x) dst4[i] = src4[i];
    for (int64_t i = (n4 << 2) + threadIdx.x; i < nwords; i += blockDim.x) sbm[i] = fbm[i];
    __syncthreads();
    fbm = sbm;
  }
  const int ln = lane_id();
  unsigned long long mf = 0, mu = 0;
  for (int64_t base = gwarp() * kWarp; base < n; base += nwarps() * kWarp) {
    const int64_t w = base + ln;
    bool found = false;
    if (w < n && dist[w] == kUnreached) {
      const int64_t e1 = g.in_rowptr[w + 1];
      for (int64_t e = g.in_rowptr[w]; e < e1; ++e) {
        const int32_t v = g.in_colidx[e];
        if ((fbm[v >> 5] >> (v & 31)) & 1u) {
          found = true;
          break;
        }
      }
    }
    const unsigned bal = __ballot_sync(kFull, found);
    if (ln == 0) nbm[base >> 5] = bal;
    if (found) {
      dist[w] = nl;
      mf += static_cast<unsigned long long>(g.rowptr[w + 1] - g.rowptr[w]);
      mu += static_cast<unsigned long long>(g.in_rowptr[w + 1] - g.in_rowptr[w]);
    }
    const unsigned long long slot = warp_append(found, &c->tail);
    if (found) b.queue[slot] = static_cast<int32_t>(w);
  }
  mf = warp_sum_u64(mf);
  mu = warp_sum_u64(mu);
  if (ln == 0) {
    if (mf) atomicAdd(&c->mf, mf);
    if (mu) atomicAdd(&c->mu_done, mu);
  }
}

__global__ void k_bfs_advance(BatchCtl* c) {
  if (c->tail == c->hi) {
    c->done = 1;
    c->maxlevel = c->level;
    c->mf_cur = 0;
    return;
  }
  c->lo = c->hi;
  c->hi = c->tail;
  c->level += 1;
  c->mf_cur = c->mf;
  c->mf = 0;
}

// _bfs_parents (src/traversals/bfs.jl:40-66) visits each level in sorted
// vertex order and gives a newly reached vertex the first level vertex that
// lists it, i.e. the smallest in-neighbour one level closer; the source is
// its own parent, unreached vertices get -1 (0 in 1-based ids).  One warp
// per vertex scans its in-list (sorted ascending) for the first neighbour at
// distance d - 1.
__global__ void __launch_bounds__(256) k_bfs_parents(DevGraph g, const int32_t* dist,
                                                     int32_t* parents) {
  const int ln = lane_id();
  for (long long v = gwarp(); v < g.n; v += nwarps()) {
    const int32_t d = dist[v];
    if (d == kUnreached || d <= 0) {
      if (ln == 0) parents[v] = d == 0 ? static_cast<int32_t>(v) : -1;
      continue;
    }
    const int64_t e0 = g.in_rowptr[v], e1 = g.in_rowptr[v + 1];
    int32_t p = -1;
    for (int64_t e = e0; e < e1; e += kWarp) {
      const int64_t idx = e + ln;
      int32_t u = 0;
      bool hit = false;
      if (idx < e1) {
        u = g.in_colidx[idx];
        hit = dist[u] == d - 1;
      }
      const unsigned bal = __ballot_sync(kFull, hit);
      if (bal) {
        p = __shfl_sync(kFull, u, __ffs(bal) - 1);
        break;
      }
    }
    if (ln == 0) parents[v] = p;
  }
}

__global__ void k_scatter_i32(int32_t* p, const int32_t* idx, int64_t count, int32_t value) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    p[idx[i]] = value;
}

}  // namespace

int bfs_configure(size_t max_dyn_smem) {
  cudaFuncSetAttribute(k_bfs_bu<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       static_cast<int>(max_dyn_smem));
  return 0;
}

int bfs_init(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const BfsBuffers& b,
             const int32_t* src, int64_t nsrc, int32_t* dist) {
  const int64_t nwords = (g.n + 31) >> 5;
  cudaMemsetAsync(b.bm[0], 0, static_cast<size_t>(nwords) * 4, s);
  cudaMemsetAsync(b.bm[1], 0, static_cast<size_t>(nwords) * 4, s);
  k_bfs_ctl_reset<<<1, 1, 0, s>>>(b.ctl);
  int launches = 1;
  if (nsrc > 0) {
    const int grid = static_cast<int>(std::min<int64_t>((nsrc + 255) / 256, c.grid));
    k_bfs_seed<<<grid, 256, 0, s>>>(g, b, src, nsrc, dist);
    ++launches;
  }
  k_bfs_seed_done<<<1, 1, 0, s>>>(b.ctl);
  return launches + 1;
}

int bfs_topdown(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const BfsBuffers& b,
                int32_t* dist) {
  const int64_t nwords = (g.n + 31) >> 5;
  k_bfs_clear_next<<<c.grid, c.block, 0, s>>>(b, nwords);
  k_bfs_td<<<c.grid, c.block, 0, s>>>(g, b, dist);
  if (!b.large) return 2;
  k_bfs_td_large<<<c.grid, c.block, 0, s>>>(g, b, dist);
  return 3;
}

int bfs_bottomup(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const BfsBuffers& b,
                 int32_t* dist, int stage_smem) {
  const int64_t nwords = (g.n + 31) >> 5;
  if (stage_smem) {
    const size_t bytes = static_cast<size_t>((nwords + 3) & ~int64_t(3)) * 4;
    // one resident 1024-thread block per SM: the bitmap is staged once per SM
    k_bfs_bu<true><<<c.sms, 1024, bytes, s>>>(g, b, dist);
  } else {
    k_bfs_bu<false><<<c.grid, c.block, 0, s>>>(g, b, dist);
  }
  return 1;
}

int bfs_parents(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const int32_t* dist,
                int32_t* parents) {
  k_bfs_parents<<<c.grid, c.block, 0, s>>>(g, dist, parents);
  return 1;
}

int scatter_i32(const LaunchCfg& c, cudaStream_t s, int32_t* p, const int32_t* idx, int64_t count,
                int32_t value) {
  if (count <= 0) return 0;
  k_scatter_i32<<<c.grid, c.block, 0, s>>>(p, idx, count, value);
  return 1;
}

int bfs_advance(cudaStream_t s, const BfsBuffers& b) {
  k_bfs_advance<<<1, 1, 0, s>>>(b.ctl);
  return 1;
}

}  // namespace lgbc
