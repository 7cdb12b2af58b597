// bfs.cu -- direction-optimising level-synchronous BFS for gdistances.
//
// Replaces gdistances! (src/traversals/bfs.jl:95-124) and its threaded
// variant (src/Parallel/traversals/gdistances.jl:36-116): every source gets
// level 0, every other vertex the level at which the BFS first reaches it,
// INT32_MAX where nothing reaches it.  The per-level sort of the reference
// (bfs.jl:121) only fixes visiting order and does not change any distance.
//
// Top-down levels expand the frontier queue over out-edges (one warp per
// frontier vertex, atomicCAS on the distance claims a vertex once).
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

// Zero the bitmap that the coming top-down level fills with atomicOr.
__global__ void k_bfs_clear_next(BfsBuffers b, int64_t nwords) {
  uint32_t* nbm = bm_at(b, b.ctl->level + 1);
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < nwords;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    nbm[i] = 0u;
}

__global__ void __launch_bounds__(256) k_bfs_td(DevGraph g, BfsBuffers b, int32_t* dist) {
  BatchCtl* c = b.ctl;
  const unsigned long long lo = c->lo, hi = c->hi;
  const int32_t nl = c->level + 1;
  uint32_t* nbm = bm_at(b, nl);
  const int ln = lane_id();
  unsigned long long mf = 0, mu = 0;
  for (unsigned long long i = lo + gwarp(); i < hi; i += nwarps()) {
    const int32_t v = b.queue[i];
    const int64_t e0 = g.rowptr[v], e1 = g.rowptr[v + 1];
    for (int64_t e = e0; e < e1; e += kWarp) {
      const int64_t idx = e + ln;
      bool app = false;
      int32_t w = 0;
      if (idx < e1) {
        w = g.colidx[idx];
        if (dist[w] == kUnreached && atomicCAS(dist + w, kUnreached, nl) == kUnreached) {
          app = true;
          atomicOr(nbm + (w >> 5), 1u << (w & 31));
          mf += static_cast<unsigned long long>(g.rowptr[w + 1] - g.rowptr[w]);
          mu += static_cast<unsigned long long>(g.in_rowptr[w + 1] - g.in_rowptr[w]);
        }
      }
      const unsigned long long slot = warp_append(app, &c->tail);
      if (app) b.queue[slot] = w;
    }
  }
  mf = warp_sum_u64(mf);
  mu = warp_sum_u64(mu);
  if (ln == 0) {
    if (mf) atomicAdd(&c->mf, mf);
    if (mu) atomicAdd(&c->mu_done, mu);
  }
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
  return 2;
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
