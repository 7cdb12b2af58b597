// learned.cu -- kernels of the learned source proposal for sampled betweenness:
// structural features (degree, core number, neighbour statistics), the
// 4 -> 64 -> 64 -> 1 MLP (BF16 weights, FP32 accumulation) forward, backward
// and Adam update, and the softmax proposal with inverse-CDF sampling.
//
// None of this has a counterpart in LightGraphs.jl except core_number
// (src/degeneracy.jl:38-80), which is computed here as the fixed point of the
// neighbourhood h-index operator (Lu, Zhou, Zhang & Stanley, "The H-index of a
// network node and its relation to degree and coreness", Nat. Commun. 2016):
// starting from the degrees, every vertex repeatedly takes the h-index of its
// neighbours' values; the values only decrease and stop exactly at the core
// numbers that the reference's bin-sort peeling returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "lgbc_kernels.h"

namespace lgbc {
namespace {

__device__ __forceinline__ long long gwarp() {
  return (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
}
__device__ __forceinline__ long long nwarps() {
  return (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
}

// ---------------------------------------------------------------------------
// Degrees and core numbers
// ---------------------------------------------------------------------------

// For a digraph the core decomposition counts every arc at both ends
// (degree = out + in, src/degeneracy.jl:41,63-96), so a vertex's neighbour
// multiset is its out-list followed by its in-list; an undirected graph's
// in-lists alias its out-lists and only those are walked.
__device__ __forceinline__ bool is_digraph(const DevGraph& g) { return g.in_colidx != g.colidx; }

// deg[v] = neighbour-list entries of v other than v itself; *loops |= 1 when
// v has a self-loop.  One warp per vertex.
__global__ void __launch_bounds__(256) k_core_degree(DevGraph g, int32_t* deg, int* loops) {
  const int ln = lane_id();
  const bool dir = is_digraph(g);
  for (long long v = gwarp(); v < g.n; v += nwarps()) {
    const int64_t e0 = g.rowptr[v], e1 = g.rowptr[v + 1];
    int64_t total = e1 - e0;
    int self = 0;
    for (int64_t e = e0 + ln; e < e1; e += kWarp) self += g.colidx[e] == v ? 1 : 0;
    if (dir) {
      const int64_t i0 = g.in_rowptr[v], i1 = g.in_rowptr[v + 1];
      total += i1 - i0;
      for (int64_t e = i0 + ln; e < i1; e += kWarp) self += g.in_colidx[e] == v ? 1 : 0;
    }
    self = __reduce_add_sync(kFull, self);
    if (ln == 0) {
      deg[v] = static_cast<int32_t>(total - self);
      if (self) atomicOr(loops, 1);
    }
  }
}

// ---- h-index passes ------------------------------------------------------------
// One pass computes, for every vertex of the list (all vertices at first), the
// h-index of its neighbours' values -- the largest h <= c (its own value) with
// #{neighbour entries u != v : core[u] >= h} >= h -- and lowers core[v] to it.
// Updates are in place; a value read while a neighbour is being lowered is at
// least that neighbour's core number, so every stored value stays >= the core
// number.  Each lowered vertex is logged with its old value; after the pass,
// k_core_flag flags the neighbours u whose count at their own value the drop
// can have changed: lo < core[u] <= c_old (a neighbour that did not count for
// u before, or still counts, cannot change u's h-index).  Only flagged
// vertices are searched again; a pass that lowers nothing is the fixed point,
// the core numbers.
struct CoreLog {
  unsigned long long* count;  // lowered vertices this pass
  int32_t* v;                 // n entries: the vertex
  int32_t* old;               // n entries: its value before the pass
};

// A vertex with at most kCoreCached neighbour entries keeps their values
// (capped at c) in registers, entry k * 32 + lane in slot k of that lane, so
// the search reads memory once; larger lists go to k_core_pass_large.
constexpr int kCoreSlots = 8;
constexpr int kCoreCached = kCoreSlots * kWarp;
// A vertex with at most kCoreThread entries is searched by one thread.
constexpr int kCoreThread = 16;

__device__ __forceinline__ int core_entries(const DevGraph& g, int32_t v) {
  int64_t d = g.rowptr[v + 1] - g.rowptr[v];
  if (is_digraph(g)) d += g.in_rowptr[v + 1] - g.in_rowptr[v];
  return d > kCoreCached ? kCoreCached + 1 : static_cast<int>(d);
}

// Entry j of v's out-list followed by its in-list (a digraph counts every arc
// at both ends); -1 past the end.
__device__ __forceinline__ int32_t core_entry(const DevGraph& g, int32_t v, int64_t o0, int64_t n0,
                                              int64_t j) {
  if (j < n0) return g.colidx[o0 + j];
  if (!is_digraph(g)) return -1;
  const int64_t k = g.in_rowptr[v] + (j - n0);
  return k < g.in_rowptr[v + 1] ? g.in_colidx[k] : -1;
}

// One thread: values counted down from min(c, entries).  Returns the new value.
__device__ __forceinline__ int32_t core_search_thread(const DevGraph& g, int32_t v, int32_t c,
                                                      int ent, const int32_t* core) {
  const int64_t o0 = g.rowptr[v], n0 = g.rowptr[v + 1] - o0;
  int32_t x[kCoreThread];
#pragma unroll
  for (int k = 0; k < kCoreThread; ++k) {
    x[k] = -1;
    if (k < ent) {
      const int32_t u = core_entry(g, v, o0, n0, k);
      if (u >= 0 && u != v) {
        const int32_t cu = core[u];
        x[k] = cu < c ? cu : c;
      }
    }
  }
  int h = c < ent ? c : ent;
  for (; h > 0; --h) {
    int cnt = 0;
#pragma unroll
    for (int k = 0; k < kCoreThread; ++k) cnt += x[k] >= h ? 1 : 0;
    if (cnt >= h) break;
  }
  return h;
}

// One warp, values in registers: count(c), then a binary search in
// [count(c), c - 1] with warp sums.  Returns the new value (c: unchanged).
__device__ __forceinline__ int32_t core_search_warp(const DevGraph& g, int32_t v, int32_t c,
                                                    const int32_t* core) {
  const int ln = lane_id();
  const int64_t o0 = g.rowptr[v], n0 = g.rowptr[v + 1] - o0;
  int32_t x[kCoreSlots];
#pragma unroll
  for (int k = 0; k < kCoreSlots; ++k) {
    x[k] = -1;
    const int32_t u = core_entry(g, v, o0, n0, static_cast<int64_t>(k) * kWarp + ln);
    if (u >= 0 && u != v) {
      const int32_t cu = core[u];
      x[k] = cu < c ? cu : c;
    }
  }
  auto count = [&](int32_t h) {
    int cnt = 0;
#pragma unroll
    for (int k = 0; k < kCoreSlots; ++k) cnt += x[k] >= h ? 1 : 0;
    return static_cast<int>(__reduce_add_sync(kFull, static_cast<unsigned>(cnt)));
  };
  const int cnt = count(c);
  if (cnt >= c) return c;
  int lo = cnt, hi = c - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (count(mid) >= mid) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ void core_log(const CoreLog& lg, unsigned long long at, int32_t v,
                                         int32_t old) {
  lg.v[at] = v;
  lg.old[at] = old;
}

// One pass: lane j of a warp takes list entry base + j.  Vertices with at
// most kCoreThread entries are searched by their own lane; the others, one at
// a time, by the whole warp, or deferred to `large` (more than kCoreCached
// entries) for k_core_pass_large.
__global__ void __launch_bounds__(256) k_core_pass(DevGraph g, const int32_t* list, long long nlist,
                                                  int32_t* core, CoreLog lg, int32_t* large,
                                                  unsigned long long* nlarge) {
  const int ln = lane_id();
  for (long long base = gwarp() * kWarp; base < nlist; base += nwarps() * kWarp) {
    const long long i = base + ln;
    int32_t v = 0, c = 0;
    int ent = 0;
    if (i < nlist) {
      v = list ? list[i] : static_cast<int32_t>(i);
      c = core[v];
      if (c > 0) ent = core_entries(g, v);
    }
    int32_t h = c;
    if (c > 0 && ent <= kCoreThread) h = core_search_thread(g, v, c, ent, core);
    const bool lowered = h < c;
    if (lowered) core[v] = h;
    const unsigned long long at = warp_append(lowered, lg.count);
    if (lowered) core_log(lg, at, v, c);
    unsigned rest = __ballot_sync(kFull, c > 0 && ent > kCoreThread);
    while (rest) {
      const int j = __ffs(rest) - 1;
      rest &= rest - 1u;
      const int32_t vj = __shfl_sync(kFull, v, j);
      const int32_t cj = __shfl_sync(kFull, c, j);
      const int entj = __shfl_sync(kFull, ent, j);
      if (entj > kCoreCached) {
        if (ln == 0) large[atomicAdd(nlarge, 1ull)] = vj;
        continue;
      }
      const int32_t hj = core_search_warp(g, vj, cj, core);
      if (hj < cj && ln == 0) {
        core[vj] = hj;
        core_log(lg, atomicAdd(lg.count, 1ull), vj, cj);
      }
    }
  }
}

// The vertices with more than kCoreCached neighbour entries (the hubs): one
// block per vertex.  One pass over the list builds a histogram of the
// neighbours' values capped at cap = min(c, kCoreHist) in shared memory, from
// whose suffix sums S(h) = #{core[u] >= h} the largest h <= cap with
// S(h) >= h is read directly; only an h-index above kCoreHist falls back to a
// binary search with one list pass per probe.
constexpr int kCoreHist = 1024;

__device__ __forceinline__ int block_sum_int(int x, int* red) {
  x = static_cast<int>(__reduce_add_sync(kFull, static_cast<unsigned>(x)));
  __syncthreads();
  if (lane_id() == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  int t = 0;
  for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) t += red[w];
  return t;
}

__device__ __forceinline__ int block_count_at_least(const DevGraph& g, int32_t v, const int32_t* core,
                                                    int32_t h, int* red) {
  int c = 0;
  for (int64_t e = g.rowptr[v] + threadIdx.x; e < g.rowptr[v + 1]; e += blockDim.x) {
    const int32_t u = g.colidx[e];
    c += (u != v && core[u] >= h) ? 1 : 0;
  }
  if (is_digraph(g))
    for (int64_t e = g.in_rowptr[v] + threadIdx.x; e < g.in_rowptr[v + 1]; e += blockDim.x) {
      const int32_t u = g.in_colidx[e];
      c += (u != v && core[u] >= h) ? 1 : 0;
    }
  return block_sum_int(c, red);
}

__global__ void __launch_bounds__(256) k_core_pass_large(DevGraph g, const int32_t* large,
                                                        const unsigned long long* nlarge,
                                                        int32_t* core, CoreLog lg) {
  // lg: the hubs' own log (their neighbours are flagged by k_core_flag_large)
  __shared__ int hist[kCoreHist + 1];
  __shared__ int red[8];
  __shared__ int s_h;
  const unsigned long long nl = *nlarge;
  const bool dir = is_digraph(g);
  for (unsigned long long i = blockIdx.x; i < nl; i += gridDim.x) {
    const int32_t v = large[i];
    const int32_t c = core[v];
    const int cap = c < kCoreHist ? c : kCoreHist;
    for (int b = threadIdx.x; b <= cap; b += blockDim.x) hist[b] = 0;
    __syncthreads();
    // lanes with the same bin add their count with one atomic
    auto bin_list = [&](const int32_t* ci, int64_t e0, int64_t e1) {
      for (int64_t b0 = e0 + (threadIdx.x & ~(kWarp - 1)); b0 < e1; b0 += blockDim.x) {
        const int64_t e = b0 + lane_id();
        int bin = -1;
        if (e < e1) {
          const int32_t u = ci[e];
          if (u != v) {
            const int32_t cu = core[u];
            bin = cu < cap ? cu : cap;
          }
        }
        const unsigned peers = __match_any_sync(kFull, bin);
        if (bin >= 0 && lane_id() == __ffs(peers) - 1) atomicAdd(&hist[bin], __popc(peers));
      }
    };
    bin_list(g.colidx, g.rowptr[v], g.rowptr[v + 1]);
    if (dir) bin_list(g.in_colidx, g.in_rowptr[v], g.in_rowptr[v + 1]);
    __syncthreads();
    if (threadIdx.x < kWarp) {
      // lane j owns bins [j B, (j + 1) B) of [0, cap] (B = ceil((cap + 1) / 32))
      const int ln = threadIdx.x;
      const int B = (cap + kWarp) / kWarp;
      const int b0 = ln * B, b1 = min(b0 + B, cap + 1);
      int part = 0;
      for (int b = b0; b < b1; ++b) part += hist[b];
      int incl = part;  // suffix sum over lanes >= ln
#pragma unroll
      for (int o = 1; o < kWarp; o <<= 1) {
        const int y = __shfl_down_sync(kFull, incl, o);
        if (ln + o < kWarp) incl += y;
      }
      int S = incl - part;  // #{values >= b1}
      int best = -1;
      for (int b = b1 - 1; b >= b0 && best < 0; --b) {
        S += hist[b];
        if (S >= b) best = b;
      }
      best = static_cast<int>(__reduce_max_sync(kFull, static_cast<unsigned>(best + 1))) - 1;
      if (ln == 0) s_h = best;
    }
    __syncthreads();
    int h = s_h;  // the h-index over values capped at cap: exact when h < kCoreHist
    if (h >= kCoreHist && c > kCoreHist) {
      if (block_count_at_least(g, v, core, c, red) >= c) {
        h = c;
      } else {
        int lo = kCoreHist, hi = c - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (block_count_at_least(g, v, core, mid, red) >= mid) lo = mid; else hi = mid - 1;
        }
        h = lo;
      }
    }
    if (h < c && threadIdx.x == 0) {
      core[v] = h;
      core_log(lg, atomicAdd(lg.count, 1ull), v, c);
    }
    __syncthreads();  // hist and s_h are reused by the next vertex
  }
}

// After a pass: for each logged vertex v (value c_old -> lo), flag the
// neighbours u with lo < core[u] <= c_old.  A warp per logged vertex (lists
// of at most kCoreCached entries); k_core_flag_large gives each logged hub a
// block.
__global__ void __launch_bounds__(256) k_core_flag(DevGraph g, const int32_t* core, uint8_t* flag,
                                                  CoreLog lg) {
  const unsigned long long nlog = *lg.count;
  const int ln = lane_id();
  for (unsigned long long i = gwarp(); i < nlog; i += nwarps()) {
    const int32_t v = lg.v[i];
    const int32_t c_old = lg.old[i];
    const int32_t lo = core[v];
    for (int64_t e = g.rowptr[v] + ln; e < g.rowptr[v + 1]; e += kWarp) {
      const int32_t u = g.colidx[e];
      const int32_t cu = core[u];
      if (u != v && cu > lo && cu <= c_old) flag[u] = 1;
    }
    if (is_digraph(g))
      for (int64_t e = g.in_rowptr[v] + ln; e < g.in_rowptr[v + 1]; e += kWarp) {
        const int32_t u = g.in_colidx[e];
        const int32_t cu = core[u];
        if (u != v && cu > lo && cu <= c_old) flag[u] = 1;
      }
  }
}

__global__ void __launch_bounds__(256) k_core_flag_large(DevGraph g, const int32_t* core,
                                                        uint8_t* flag, CoreLog lg) {
  const unsigned long long nlog = *lg.count;
  for (unsigned long long i = blockIdx.x; i < nlog; i += gridDim.x) {
    const int32_t v = lg.v[i];
    const int32_t c_old = lg.old[i];
    const int32_t lo = core[v];
    for (int64_t e = g.rowptr[v] + threadIdx.x; e < g.rowptr[v + 1]; e += blockDim.x) {
      const int32_t u = g.colidx[e];
      const int32_t cu = core[u];
      if (u != v && cu > lo && cu <= c_old) flag[u] = 1;
    }
    if (is_digraph(g))
      for (int64_t e = g.in_rowptr[v] + threadIdx.x; e < g.in_rowptr[v + 1]; e += blockDim.x) {
        const int32_t u = g.in_colidx[e];
        const int32_t cu = core[u];
        if (u != v && cu > lo && cu <= c_old) flag[u] = 1;
      }
  }
}

// Gather the flagged vertices into `list` (and clear the flags).
__global__ void k_core_compact(int64_t n, uint8_t* flag, int32_t* list, unsigned long long* count) {
  const int ln = lane_id();
  for (long long base = static_cast<long long>(blockIdx.x) * blockDim.x; base < n;
       base += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long v = base + threadIdx.x;
    const bool f = v < n && flag[v];
    const unsigned bal = __ballot_sync(kFull, f);
    if (!bal) continue;
    unsigned long long at = 0;
    if (ln == 0) at = atomicAdd(count, static_cast<unsigned long long>(__popc(bal)));
    at = __shfl_sync(kFull, at, 0);
    if (f) {
      flag[v] = 0;
      list[at + __popc(bal & ((1u << ln) - 1u))] = static_cast<int32_t>(v);
    }
  }
}

// ---------------------------------------------------------------------------
// Features: (log(1 + deg), log(1 + core), mean log(1 + deg u) over the
// neighbours u, log(1 + sum of the neighbours' degrees)).  Degrees here are
// CSR row lengths (a self-loop counts once, as length(fadjlist[v])).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_features(DevGraph g, const int32_t* core, float4* feat) {
  const int ln = lane_id();
  for (long long v = gwarp(); v < g.n; v += nwarps()) {
    const int64_t e0 = g.rowptr[v], e1 = g.rowptr[v + 1];
    float sl = 0.f;
    unsigned long long sd = 0;
    for (int64_t e = e0 + ln; e < e1; e += kWarp) {
      const int32_t u = g.colidx[e];
      const int64_t du = g.rowptr[u + 1] - g.rowptr[u];
      sl += log1pf(static_cast<float>(du));
      sd += static_cast<unsigned long long>(du);
    }
    for (int o = 16; o > 0; o >>= 1) {
      sl += __shfl_xor_sync(kFull, sl, o);
      sd += __shfl_xor_sync(kFull, sd, o);
    }
    if (ln == 0) {
      const int64_t d = e1 - e0;
      float4 f;
      f.x = log1pf(static_cast<float>(d));
      f.y = log1pf(static_cast<float>(core[v]));
      f.z = d > 0 ? sl / static_cast<float>(d) : 0.f;
      f.w = log1pf(static_cast<float>(sd));
      feat[v] = f;
    }
  }
}

// ---------------------------------------------------------------------------
// MLP 4 -> 64 -> 64 -> 1 with ReLU.  Parameters (offsets in kMlp*):
//   W1[64][4], b1[64], W2[64][64] (row = output unit), b2[64], W3[64], b3.
// Weights are BF16 in device memory and widened to FP32 in shared memory;
// every product and sum is FP32.  Inputs are standardised by (x - mu) * isd.
// ---------------------------------------------------------------------------
constexpr int kH = kMlpHidden;

__device__ __forceinline__ void load_weights(const __nv_bfloat16* __restrict__ P, float* w) {
  for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) w[i] = __bfloat162float(P[i]);
  __syncthreads();
}

__device__ __forceinline__ void standardise(float4 xi, const MlpNorm& nm, float x[4]) {
  x[0] = (xi.x - nm.mu[0]) * nm.isd[0];
  x[1] = (xi.y - nm.mu[1]) * nm.isd[1];
  x[2] = (xi.z - nm.mu[2]) * nm.isd[2];
  x[3] = (xi.w - nm.mu[3]) * nm.isd[3];
}

__device__ __forceinline__ void layer1(const float* w, const float x[4], float h1[kH]) {
#pragma unroll
  for (int j = 0; j < kH; ++j) {
    float a = w[kMlpB1 + j];
    a = fmaf(w[kMlpW1 + 4 * j + 0], x[0], a);
    a = fmaf(w[kMlpW1 + 4 * j + 1], x[1], a);
    a = fmaf(w[kMlpW1 + 4 * j + 2], x[2], a);
    a = fmaf(w[kMlpW1 + 4 * j + 3], x[3], a);
    h1[j] = fmaxf(a, 0.f);
  }
}

// Pre-activation of hidden unit j of layer 2.
__device__ __forceinline__ float layer2_unit(const float* w, const float h1[kH], int j) {
  const float4* row = reinterpret_cast<const float4*>(w + kMlpW2 + kH * j);
  float a = w[kMlpB2 + j];
#pragma unroll
  for (int i = 0; i < kH / 4; ++i) {
    const float4 q = row[i];
    a = fmaf(q.x, h1[4 * i + 0], a);
    a = fmaf(q.y, h1[4 * i + 1], a);
    a = fmaf(q.z, h1[4 * i + 2], a);
    a = fmaf(q.w, h1[4 * i + 3], a);
  }
  return a;
}

__global__ void __launch_bounds__(256) k_mlp_forward(const float4* __restrict__ x, long long rows,
                                                     const __nv_bfloat16* __restrict__ P, MlpNorm nm,
                                                     float* __restrict__ y) {
  __shared__ __align__(16) float w[kMlpParamsPadded];
  load_weights(P, w);
  for (long long r = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; r < rows;
       r += static_cast<long long>(gridDim.x) * blockDim.x) {
    // keep the weights in shared memory: without this barrier the compiler
    // hoists loop-invariant weight loads out of the row loop and spills
    asm volatile("" ::: "memory");
    float xs[4], h1[kH];
    standardise(x[r], nm, xs);
    layer1(w, xs, h1);
    float out = w[kMlpB3];
#pragma unroll 2
    for (int j = 0; j < kH; ++j) out = fmaf(w[kMlpW3 + j], fmaxf(layer2_unit(w, h1, j), 0.f), out);
    y[r] = out;
  }
}

// Training forward: e[r] = yhat(x[r0 + r]) - target[r0 + r], r < B.
__global__ void __launch_bounds__(256) k_mlp_residual(const float4* __restrict__ x,
                                                      const float* __restrict__ target, long long r0,
                                                      int B, const __nv_bfloat16* __restrict__ P,
                                                      MlpNorm nm, float* __restrict__ e) {
  __shared__ __align__(16) float w[kMlpParamsPadded];
  load_weights(P, w);
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < B; r += gridDim.x * blockDim.x) {
    asm volatile("" ::: "memory");
    float xs[4], h1[kH];
    standardise(x[r0 + r], nm, xs);
    layer1(w, xs, h1);
    float out = w[kMlpB3];
#pragma unroll 2
    for (int j = 0; j < kH; ++j) out = fmaf(w[kMlpW3 + j], fmaxf(layer2_unit(w, h1, j), 0.f), out);
    e[r] = out - target[r0 + r];
  }
}

// Block-wide sum of one float per thread (blockDim.x a multiple of 32).
__device__ __forceinline__ float block_sum(float v, float* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  __syncthreads();
  if (lane_id() == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float s = 0.f;
  for (int i = 0; i < static_cast<int>(blockDim.x >> 5); ++i) s += red[i];
  return s;
}

// Mean residual and loss of the batch, once per step (one block, fixed order):
// center = sum(e) / B, loss = sum((e - center)^2) / B.
__global__ void __launch_bounds__(1024) k_mlp_center(const float* __restrict__ e, int B,
                                                     float* __restrict__ center,
                                                     float* __restrict__ loss) {
  __shared__ float red[32];
  const int t = threadIdx.x;
  float s = 0.f;
  for (int r = t; r < B; r += blockDim.x) s += e[r];
  const float mean = block_sum(s, red) / static_cast<float>(B);
  float q = 0.f;
  for (int r = t; r < B; r += blockDim.x) {
    const float d = e[r] - mean;
    q += d * d;
  }
  q = block_sum(q, red);
  if (t == 0) {
    *center = mean;
    *loss = q / static_cast<float>(B);
  }
}

// Gradient of the per-batch centred squared error
//   loss = (1 / B) sum_r (e_r - mean(e))^2,   dloss / dyhat_r = 2 (e_r - mean(e)) / B
// (the softmax proposal is shift-invariant, so only relative log-masses
// within one graph matter).  Block b handles rows [b * kGradRows, ...) with
// two threads per row and writes its partial gradient to part[b][kMlpParams]
// (the batch mean comes from k_mlp_center).  Activations of the block's rows are staged
// in shared memory and the weight gradients reduced over rows there.
// dloss / da2[r][j] is not staged: it is g_r W3[j] where relu(a2[r][j]) > 0,
// else 0, recomputed from the staged relu(a2) and g.  A 64-row block holds
// 68 KB of shared memory; at two blocks per SM every thread keeps its 64-wide
// h1 and dh1 rows in registers without spilling (three blocks spill ~400 B).
constexpr int kStride = kH + 1;  // padded row stride (no bank conflicts)

// Hidden unit of step q (0..31) for half h of a row's pair of threads:
// 16-unit runs alternate between the halves, so the 32 lanes of a warp
// (16 rows x 2 halves) write 32 distinct banks of a kStride-padded row.
__device__ __forceinline__ int pair_unit(int h, int q) { return ((q >> 4) << 5) | (h << 4) | (q & 15); }

__global__ void __launch_bounds__(kGradThreads, 2) k_mlp_grad(const float4* __restrict__ x,
                                                             long long r0, int B,
                                                             const float* __restrict__ e,
                                                             const float* __restrict__ center,
                                                             const __nv_bfloat16* __restrict__ P,
                                                             MlpNorm nm, float* __restrict__ part) {
  extern __shared__ __align__(16) float sm[];
  float* w = sm;                                  // kMlpParamsPadded
  float* s_h1 = w + kMlpParamsPadded;             // [rows][kStride]
  float* s_h2 = s_h1 + kGradRows * kStride;       // relu(a2)
  float* s_d1 = s_h2 + kGradRows * kStride;       // dloss / da1
  float* s_x = s_d1 + kGradRows * kStride;        // [rows][4] standardised inputs
  float* s_g = s_x + kGradRows * 4;               // dloss / dyhat
  load_weights(P, w);
  const int t = threadIdx.x;
  const float mean = *center;

  const int rl = t >> 1, half = t & 1;
  const int r = blockIdx.x * kGradRows + rl;
  const bool live = r < B;
  float gr = 0.f;
  if (live) gr = 2.f * (e[r] - mean) / static_cast<float>(B);
  if (half == 0) s_g[rl] = gr;
  {
    float xs[4] = {0.f, 0.f, 0.f, 0.f};
    float h1[kH], dh1[kH];
    if (live) standardise(x[r0 + r], nm, xs);
    layer1(w, xs, h1);
#pragma unroll
    for (int i = 0; i < kH; ++i) dh1[i] = 0.f;
    // register indices stay compile-time: select between the halves' units
#pragma unroll
    for (int q = 0; q < kH / 2; ++q)
      s_h1[rl * kStride + pair_unit(half, q)] = half ? h1[pair_unit(1, q)] : h1[pair_unit(0, q)];
    s_x[rl * 4 + 2 * half] = half ? xs[2] : xs[0];
    s_x[rl * 4 + 2 * half + 1] = half ? xs[3] : xs[1];
    // this thread's 32 units of layer 2; the pair's dh1 halves are summed below
#pragma unroll 2
    for (int q = 0; q < kH / 2; ++q) {
      const int j = pair_unit(half, q);
      const float a = layer2_unit(w, h1, j);
      const float d2 = a > 0.f ? gr * w[kMlpW3 + j] : 0.f;
      s_h2[rl * kStride + j] = fmaxf(a, 0.f);
      const float4* row = reinterpret_cast<const float4*>(w + kMlpW2 + kH * j);
#pragma unroll
      for (int i = 0; i < kH / 4; ++i) {
        const float4 v = row[i];
        dh1[4 * i + 0] = fmaf(v.x, d2, dh1[4 * i + 0]);
        dh1[4 * i + 1] = fmaf(v.y, d2, dh1[4 * i + 1]);
        dh1[4 * i + 2] = fmaf(v.z, d2, dh1[4 * i + 2]);
        dh1[4 * i + 3] = fmaf(v.w, d2, dh1[4 * i + 3]);
      }
    }
    // the pair's two partial sums (a + b == b + a, so both threads agree)
#pragma unroll
    for (int i = 0; i < kH; ++i) dh1[i] += __shfl_xor_sync(kFull, dh1[i], 1);
#pragma unroll
    for (int q = 0; q < kH / 2; ++q) {
      const int i0 = pair_unit(0, q), i1 = pair_unit(1, q);
      const float hv = half ? h1[i1] : h1[i0], dv = half ? dh1[i1] : dh1[i0];
      s_d1[rl * kStride + pair_unit(half, q)] = hv > 0.f ? dv : 0.f;
    }
  }
  __syncthreads();

  const int rows_here = min(kGradRows, B - static_cast<int>(blockIdx.x) * kGradRows);
  float* out = part + static_cast<int64_t>(blockIdx.x) * kMlpParams;
  // dW2[j][i] = sum_r d2[r][j] h1[r][i]: thread t owns j = t / 2 and the 32
  // i's of parity t & 1 (the two halves read neighbouring banks)
  {
    const int j = t >> 1, ip = t & 1;
    const float w3 = w[kMlpW3 + j];
    float acc[32];
#pragma unroll
    for (int q = 0; q < 32; ++q) acc[q] = 0.f;
    for (int rr = 0; rr < rows_here; ++rr) {
      const float d = s_h2[rr * kStride + j] > 0.f ? s_g[rr] * w3 : 0.f;
      const float* h = s_h1 + rr * kStride + ip;
#pragma unroll
      for (int q = 0; q < 32; ++q) acc[q] = fmaf(d, h[2 * q], acc[q]);
    }
#pragma unroll
    for (int q = 0; q < 32; ++q) out[kMlpW2 + kH * j + 2 * q + ip] = acc[q];
  }
  if (t < kH) {  // dW3[j], db2[j]
    const float w3 = w[kMlpW3 + t];
    float a3 = 0.f, a2 = 0.f;
    for (int rr = 0; rr < rows_here; ++rr) {
      const float h2 = s_h2[rr * kStride + t];
      a3 = fmaf(s_g[rr], h2, a3);
      a2 += h2 > 0.f ? s_g[rr] * w3 : 0.f;
    }
    out[kMlpW3 + t] = a3;
    out[kMlpB2 + t] = a2;
  } else {  // dW1[i][f], db1[i]
    const int i = t - kH;
    float a[4] = {0.f, 0.f, 0.f, 0.f}, b = 0.f;
    for (int rr = 0; rr < rows_here; ++rr) {
      const float d = s_d1[rr * kStride + i];
#pragma unroll
      for (int f = 0; f < 4; ++f) a[f] = fmaf(d, s_x[rr * 4 + f], a[f]);
      b += d;
    }
#pragma unroll
    for (int f = 0; f < 4; ++f) out[kMlpW1 + 4 * i + f] = a[f];
    out[kMlpB1 + i] = b;
  }
  if (t == 0) {
    float b3 = 0.f;
    for (int rr = 0; rr < rows_here; ++rr) b3 += s_g[rr];
    out[kMlpB3] = b3;
  }
}

// grad[p] = sum over blocks of part[b][p] (fixed order), then optionally an
// Adam step on the FP32 master weights and their BF16 copy.
__global__ void k_mlp_reduce_adam(const float* __restrict__ part, int nblocks, float* grad,
                                  float* master, __nv_bfloat16* P, float* m1, float* m2,
                                  AdamStep st) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kMlpParams) return;
  float gsum = 0.f;
  for (int b = 0; b < nblocks; ++b) gsum += part[static_cast<int64_t>(b) * kMlpParams + p];
  if (grad) grad[p] = gsum;
  if (!master) return;
  const float a = st.beta1 * m1[p] + (1.f - st.beta1) * gsum;
  const float v = st.beta2 * m2[p] + (1.f - st.beta2) * gsum * gsum;
  m1[p] = a;
  m2[p] = v;
  const float mhat = a / st.bc1, vhat = v / st.bc2;
  const float wnew = master[p] - st.lr * mhat / (sqrtf(vhat) + st.eps);
  master[p] = wnew;
  P[p] = __float2bfloat16_rn(wnew);
}

__global__ void k_to_bf16(const float* master, __nv_bfloat16* P, int count) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < count) P[p] = __float2bfloat16_rn(master[p]);
}

// ---------------------------------------------------------------------------
// Proposal p = (1 - eps) softmax(y) + eps / n, its CDF, and sampling.
// Reductions and the scan use fixed block partitions, so results do not
// depend on scheduling.
// ---------------------------------------------------------------------------
constexpr int kScanBlock = 1024;
constexpr int kScanItems = 4;  // elements per thread
constexpr int kScanTile = kScanBlock * kScanItems;

__global__ void __launch_bounds__(kScanBlock) k_block_max(const float* y, int64_t n, float* bmax) {
  __shared__ float red[32];
  float m = -INFINITY;
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile;
  for (int q = 0; q < kScanItems; ++q) {
    const int64_t i = base + q * kScanBlock + threadIdx.x;
    if (i < n) m = fmaxf(m, y[i]);
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(kFull, m, o));
  if (lane_id() == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float r = red[0];
    for (int i = 1; i < kScanBlock / 32; ++i) r = fmaxf(r, red[i]);
    bmax[blockIdx.x] = r;
  }
}

// One block: reduce nb partial maxima into *out.
__global__ void __launch_bounds__(kScanBlock) k_max_final(const float* bmax, int64_t nb, float* out) {
  __shared__ float red[32];
  float m = -INFINITY;
  for (int64_t i = threadIdx.x; i < nb; i += kScanBlock) m = fmaxf(m, bmax[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(kFull, m, o));
  if (lane_id() == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float r = red[0];
    for (int i = 1; i < kScanBlock / 32; ++i) r = fmaxf(r, red[i]);
    *out = r;
  }
}

// Inclusive block scan of doubles (kScanBlock threads), returns the total.
__device__ __forceinline__ double block_scan(double v, double* red, double* incl) {
  const int ln = lane_id(), wid = threadIdx.x >> 5;
  double x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const double y = __shfl_up_sync(kFull, x, o);
    if (ln >= o) x += y;
  }
  if (ln == 31) red[wid] = x;
  __syncthreads();
  if (wid == 0) {
    double s = ln < kScanBlock / 32 ? red[ln] : 0.0;
    for (int o = 1; o < 32; o <<= 1) {
      const double y = __shfl_up_sync(kFull, s, o);
      if (ln >= o) s += y;
    }
    red[ln] = s;
  }
  __syncthreads();
  *incl = x + (wid > 0 ? red[wid - 1] : 0.0);
  const double total = red[kScanBlock / 32 - 1];
  __syncthreads();
  return total;
}

// e[i] = exp(y[i] - ymax) in FP64; per-tile sums.
__global__ void __launch_bounds__(kScanBlock) k_exp_tile(const float* y, int64_t n, const float* ymax,
                                                         double* e, double* tsum) {
  __shared__ double red[32];
  const double m = static_cast<double>(*ymax);
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile + static_cast<int64_t>(threadIdx.x) * kScanItems;
  double s = 0.0;
  for (int q = 0; q < kScanItems; ++q) {
    const int64_t i = base + q;
    if (i < n) {
      const double v = exp(static_cast<double>(y[i]) - m);
      e[i] = v;
      s += v;
    }
  }
  double incl;
  const double total = block_scan(s, red, &incl);
  if (threadIdx.x == 0) tsum[blockIdx.x] = total;
}

// One block: exclusive scan of the nb tile sums in place, total in *tot.
__global__ void __launch_bounds__(kScanBlock) k_scan_tiles(double* tsum, int64_t nb, double* tot) {
  __shared__ double red[32];
  double carry = 0.0;
  for (int64_t b0 = 0; b0 < nb; b0 += kScanBlock) {
    const int64_t i = b0 + threadIdx.x;
    const double v = i < nb ? tsum[i] : 0.0;
    double incl;
    const double total = block_scan(v, red, &incl);
    if (i < nb) tsum[i] = carry + incl - v;
    carry += total;
  }
  if (threadIdx.x == 0) *tot = carry;
}

// p[i] = (1 - eps) e[i] / Z + eps / n and cdf[i] = inclusive prefix of p,
// built from the softmax prefix (1 - eps) E_i / Z + eps (i + 1) / n so that
// cdf[n - 1] = 1 up to rounding.
__global__ void __launch_bounds__(kScanBlock) k_prob_cdf(const double* e, int64_t n, const double* toff,
                                                         const double* Z, double eps, double* p,
                                                         double* cdf) {
  __shared__ double red[32];
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile + static_cast<int64_t>(threadIdx.x) * kScanItems;
  double loc[kScanItems];
  double s = 0.0;
  for (int q = 0; q < kScanItems; ++q) {
    const int64_t i = base + q;
    loc[q] = i < n ? e[i] : 0.0;
    s += loc[q];
  }
  double incl;
  block_scan(s, red, &incl);
  double run = toff[blockIdx.x] + incl - s;
  const double zinv = 1.0 / *Z, a = 1.0 - eps, u = eps / static_cast<double>(n);
  for (int q = 0; q < kScanItems; ++q) {
    const int64_t i = base + q;
    if (i < n) {
      run += loc[q];
      p[i] = a * loc[q] * zinv + u;
      cdf[i] = a * run * zinv + u * static_cast<double>(i + 1);
    }
  }
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Sample i: u in [0, cdf[n - 1]); the vertex is the first index with
// cdf > u; weight 1 / (k p).  Independent draws take u from SplitMix64(seed,
// i); systematic draws take u = (i + U) / k of the total with one U from the
// seed, so vertex s is drawn floor or ceil of k p_s times (Madow 1949), still
// k p_s on average, which keeps the weighted sum unbiased.
__global__ void k_sample(const double* cdf, const double* p, int64_t n, int64_t k, uint64_t seed,
                         bool systematic, int32_t* src, double* w) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= k) return;
  double u;
  if (systematic) {
    const double U = static_cast<double>(splitmix64(seed ^ 0x5851F42D4C957F2Dull) >> 11) * 0x1.0p-53;
    u = fmin((static_cast<double>(i) + U) / static_cast<double>(k), 1.0 - 0x1.0p-53) * cdf[n - 1];
  } else {
    const uint64_t r = splitmix64(seed ^ splitmix64(static_cast<uint64_t>(i)));
    u = static_cast<double>(r >> 11) * 0x1.0p-53 * cdf[n - 1];
  }
  int64_t lo = 0, hi = n - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (cdf[mid] > u) hi = mid; else lo = mid + 1;
  }
  src[i] = static_cast<int32_t>(lo);
  w[i] = 1.0 / (static_cast<double>(k) * p[lo]);
}

}  // namespace

// ---------------------------------------------------------------------------
// Host wrappers
// ---------------------------------------------------------------------------
int core_degree(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, int32_t* deg, int* loops) {
  k_core_degree<<<c.grid, c.block, 0, s>>>(g, deg, loops);
  return 1;
}

int core_pass(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const int32_t* list,
              int64_t nlist, int32_t* core, uint8_t* flag, const CorePassBuffers& b) {
  if (nlist <= 0) return 0;
  const int64_t want = (nlist + 255) / 256;  // a warp takes 32 entries, a block 256
  const int grid = static_cast<int>(want < c.grid ? want : c.grid);
  const CoreLog lg{b.changed, b.log_v, b.log_old};
  const CoreLog lh{b.changed_hubs, b.hub_v, b.hub_old};
  cudaMemsetAsync(b.changed, 0, sizeof(unsigned long long), s);
  cudaMemsetAsync(b.changed_hubs, 0, sizeof(unsigned long long), s);
  cudaMemsetAsync(b.nlarge, 0, sizeof(unsigned long long), s);
  k_core_pass<<<grid, 256, 0, s>>>(g, list, nlist, core, lg, b.large, b.nlarge);
  k_core_pass_large<<<c.grid, 256, 0, s>>>(g, b.large, b.nlarge, core, lh);
  k_core_flag<<<c.grid, 256, 0, s>>>(g, core, flag, lg);
  k_core_flag_large<<<c.grid, 256, 0, s>>>(g, core, flag, lh);
  return 4;
}

int core_compact(const LaunchCfg& c, cudaStream_t s, int64_t n, uint8_t* flag, int32_t* list,
                 unsigned long long* count) {
  k_core_compact<<<c.grid, c.block, 0, s>>>(n, flag, list, count);
  return 1;
}

int features(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const int32_t* core,
             float4* feat) {
  k_features<<<c.grid, c.block, 0, s>>>(g, core, feat);
  return 1;
}

int mlp_forward(const LaunchCfg& c, cudaStream_t s, const float4* x, int64_t rows,
                const __nv_bfloat16* P, const MlpNorm& nm, float* y) {
  if (rows <= 0) return 0;
  const int64_t want = (rows + 255) / 256;
  const int grid = static_cast<int>(want < c.sms * 8 ? want : c.sms * 8);
  k_mlp_forward<<<grid, 256, 0, s>>>(x, rows, P, nm, y);
  return 1;
}

size_t mlp_grad_smem() {
  return sizeof(float) * (kMlpParamsPadded + 3 * kGradRows * kStride + kGradRows * 4 + kGradRows);
}

int mlp_configure() {
  const cudaError_t e = cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(mlp_grad_smem()));
  return e == cudaSuccess ? 0 : -1;
}

int mlp_train_step(cudaStream_t s, const float4* x, const float* target, int64_t r0, int B,
                   const __nv_bfloat16* P, const MlpNorm& nm, float* e, float* center,
                   float* part, float* loss, float* grad, float* master, __nv_bfloat16* Pw,
                   float* m1, float* m2, const AdamStep& st) {
  const int nb = (B + kGradRows - 1) / kGradRows;
  k_mlp_residual<<<(B + 255) / 256, 256, 0, s>>>(x, target, r0, B, P, nm, e);
  k_mlp_center<<<1, 1024, 0, s>>>(e, B, center, loss);
  k_mlp_grad<<<nb, kGradThreads, mlp_grad_smem(), s>>>(x, r0, B, e, center, P, nm, part);
  k_mlp_reduce_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(part, nb, grad, master, Pw, m1, m2, st);
  return 4;
}

int mlp_to_bf16(cudaStream_t s, const float* master, __nv_bfloat16* P) {
  k_to_bf16<<<(kMlpParams + 255) / 256, 256, 0, s>>>(master, P, kMlpParams);
  return 1;
}

int64_t proposal_tiles(int64_t n) { return (n + kScanTile - 1) / kScanTile; }

int proposal_build(cudaStream_t s, const float* y, int64_t n, double eps, float* fscratch,
                   double* e, double* tsum, double* scal, double* p, double* cdf) {
  const int64_t nb = proposal_tiles(n);
  float* bmax = fscratch;          // nb
  float* ymax = fscratch + nb;     // 1
  k_block_max<<<static_cast<unsigned>(nb), kScanBlock, 0, s>>>(y, n, bmax);
  k_max_final<<<1, kScanBlock, 0, s>>>(bmax, nb, ymax);
  k_exp_tile<<<static_cast<unsigned>(nb), kScanBlock, 0, s>>>(y, n, ymax, e, tsum);
  k_scan_tiles<<<1, kScanBlock, 0, s>>>(tsum, nb, scal);
  k_prob_cdf<<<static_cast<unsigned>(nb), kScanBlock, 0, s>>>(e, n, tsum, scal, eps, p, cdf);
  return 5;
}

int proposal_sample(cudaStream_t s, const double* cdf, const double* p, int64_t n, int64_t k,
                    uint64_t seed, bool systematic, int32_t* src, double* w) {
  if (k <= 0) return 0;
  k_sample<<<static_cast<unsigned>((k + 255) / 256), 256, 0, s>>>(cdf, p, n, k, seed, systematic,
                                                                  src, w);
  return 1;
}

}  // namespace lgbc
