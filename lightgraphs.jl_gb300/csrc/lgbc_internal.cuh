// lgbc_internal.cuh -- shared device helpers for the lgbc CUDA library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lgbc {

constexpr int kWarp = 32;
constexpr int kMaxLanes = 64;            // sources per one-word multi-source batch
constexpr int kMaxWords = 4;             // 64-bit lane words per vertex in a wide batch
constexpr int kWideLanes = 64 * kMaxWords;  // sources per widest (four-word) batch

// Lane words of a batch of nl lanes: 1, 2 or 4 (three-word batches round up).
constexpr int lane_words(int nl) { return nl > 2 * kMaxLanes ? 4 : (nl > kMaxLanes ? 2 : 1); }
constexpr int32_t kUnreached = INT32_MAX;
constexpr unsigned kFull = 0xffffffffu;

// Device view of a graph: out-CSR and in-CSR (the same arrays for an
// undirected graph, whose fadjlist is also its badjlist).
struct DevGraph {
  int64_t n;
  int64_t nnz;
  const int64_t* rowptr;
  const int32_t* colidx;
  const int64_t* in_rowptr;
  const int32_t* in_colidx;
};

// Per-batch control block, resident in device memory.  Kernels read the
// current frontier range from it, so a level's launches are identical from
// level to level and the host never has to patch arguments.
struct BatchCtl {
  unsigned long long lo;        // current frontier Q_L = list[lo, hi)
  unsigned long long hi;
  unsigned long long tail;      // append cursor for Q_{L+1}
  unsigned long long mf;        // out-edges of the entries appended this level
  unsigned long long mf_cur;    // out-edges of the current frontier Q_L
  unsigned long long mu_done;   // in-edges of vertices every lane has visited
  unsigned long long cap;       // list capacity (entries)
  int level;                    // L (forward: frontier level; backward: level swept)
  int maxlevel;                 // deepest non-empty level (set when the forward ends)
  int done;                     // forward finished (Q_{L+1} empty)
  int overflow_list;            // list capacity exceeded (host grows + replays)
  int overflow_sigma;           // path counts may exceed 2^64 (host replays in FP64)
  int mode;                     // 0 = top-down, 1 = bottom-up (for the next level)
  unsigned long long sigma_max;   // largest path count stored this level
  unsigned long long sigma_limit; // (2^64 - 1) / (max in-degree + 1): a level whose
                                  // counts stay <= this cannot overflow the next
  unsigned long long td_levels;   // levels expanded top-down / bottom-up by a
  unsigned long long bu_levels;   //   device-driven level loop
  int runaway;                    // a device-driven loop reached its level cap
  // lanes present in the current frontier Q_L (a superset is allowed): a lane
  // outside it discovers nothing at level L + 1, so bottom-up scans skip it
  unsigned long long front_union[kMaxWords];
  unsigned long long next_union[kMaxWords];  // lanes of Q_{L+1}, accumulated after its appends
  unsigned long long large;     // single-source BFS: high-degree frontier vertices deferred this level
};

// ---------------------------------------------------------------------------
// Warp helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ int lane_id() { return threadIdx.x & (kWarp - 1); }

__device__ __forceinline__ uint64_t shfl_u64(uint64_t x, int src) {
  uint32_t lo = static_cast<uint32_t>(x), hi = static_cast<uint32_t>(x >> 32);
  lo = __shfl_sync(kFull, lo, src);
  hi = __shfl_sync(kFull, hi, src);
  return (static_cast<uint64_t>(hi) << 32) | lo;
}

__device__ __forceinline__ uint64_t warp_or_u64(uint64_t x) {
  uint32_t lo = __reduce_or_sync(kFull, static_cast<uint32_t>(x));
  uint32_t hi = __reduce_or_sync(kFull, static_cast<uint32_t>(x >> 32));
  return (static_cast<uint64_t>(hi) << 32) | lo;
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = shfl_u64(x, lane_id() ^ o);
    x = y > x ? y : x;
  }
  return x;
}

// 32 x 32 bit-matrix transpose across a warp: thread t enters with row t
// (bit j = element (t, j)) and leaves with column t (bit j = element (j, t)).
// Recursive block swap (Hacker's Delight 7-3) with one shuffle per level.
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t a) {
  const int ln = threadIdx.x & 31;
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const uint32_t m = s == 16 ? 0x0000FFFFu : s == 8 ? 0x00FF00FFu : s == 4 ? 0x0F0F0F0Fu
                     : s == 2 ? 0x33333333u : 0x55555555u;
    const uint32_t x = __shfl_xor_sync(0xffffffffu, a, s);
    a = (ln & s) ? ((a & ~m) | ((x & ~m) >> s)) : ((a & m) | ((x & m) << s));
  }
  return a;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += shfl_u64(x, lane_id() ^ o);
  return x;
}

// Warp-aggregated append: every lane with `want` gets a distinct slot from
// *cursor; returns the slot (undefined for lanes without `want`).
__device__ __forceinline__ unsigned long long warp_append(bool want,
                                                          unsigned long long* cursor) {
  unsigned ballot = __ballot_sync(kFull, want);
  unsigned long long base = 0;
  int leader = __ffs(ballot) - 1;
  if (ballot != 0 && lane_id() == leader)
    base = atomicAdd(cursor, static_cast<unsigned long long>(__popc(ballot)));
  base = shfl_u64(base, leader < 0 ? 0 : leader);
  return base + __popc(ballot & ((1u << lane_id()) - 1u));
}

// ---------------------------------------------------------------------------
// Double-float ("df") arithmetic: a value is hi + lo with |lo| <= ulp(hi)/2,
// about 48 significant bits.  GB300 executes FP64 at a small fraction of its
// FP32 rate, so the dependency sweep keeps its per-edge sums in df built from
// FP32 operations (Dekker 1971 / Knuth TAOCP vol. 2 error-free transforms;
// Shewchuk 1997).  Every operand on this path is non-negative, so the
// accumulated relative error stays near levels * 2^-47.
// Compile WITHOUT fast-math: these transforms rely on IEEE round-to-nearest.
// ---------------------------------------------------------------------------
struct df32 {
  float hi, lo;
};

__device__ __forceinline__ df32 df_make(float hi, float lo) { return df32{hi, lo}; }

// Knuth TwoSum: s + e == a + b exactly.
__device__ __forceinline__ df32 two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df32{s, e};
}

// Dekker FastTwoSum, valid when |a| >= |b|.
__device__ __forceinline__ df32 fast_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return df32{s, e};
}

__device__ __forceinline__ df32 df_add(df32 a, df32 b) {
  df32 s = two_sum(a.hi, b.hi);
  float lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, lo);
}

__device__ __forceinline__ df32 df_add_f(df32 a, float b) {
  df32 s = two_sum(a.hi, b);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}

// Product with the error of hi*hi recovered exactly by an FMA.
__device__ __forceinline__ df32 df_mul(df32 a, df32 b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

// Quotient: q1 = a.hi / b.hi, then one correction step on the df remainder.
__device__ __forceinline__ df32 df_div(df32 a, df32 b) {
  float q1 = __fdiv_rn(a.hi, b.hi);
  // r = a - q1 * b, computed with exact products
  float p = __fmul_rn(q1, b.hi);
  float pe = __fmaf_rn(q1, b.hi, -p);
  pe = __fmaf_rn(q1, b.lo, pe);
  df32 r = two_sum(a.hi, -p);
  r.lo = __fadd_rn(__fsub_rn(r.lo, pe), a.lo);
  float rr = __fadd_rn(r.hi, r.lo);
  float q2 = __fdiv_rn(rr, b.hi);
  return fast_two_sum(q1, q2);
}

// Exact-as-possible conversion of a path count to df (exact below 2^48).
__device__ __forceinline__ df32 df_from_u64(unsigned long long x) {
  float hi = __ull2float_rn(x);
  // x - hi fits in int64 because |x - hi| <= ulp(hi)/2 < 2^40 for x < 2^64
  long long rem = static_cast<long long>(x - static_cast<unsigned long long>(
                                                 __float2ull_rn(hi)));
  if (hi >= 1.8446744e19f) rem = 0;  // hi rounded up to 2^64: keep hi only
  float lo = __ll2float_rn(rem);
  return fast_two_sum(hi, lo);
}

__device__ __forceinline__ double df_to_double(df32 a) {
  return static_cast<double>(a.hi) + static_cast<double>(a.lo);
}

__device__ __forceinline__ df32 shfl_df(df32 x, int src) {
  return df32{__shfl_sync(kFull, x.hi, src), __shfl_sync(kFull, x.lo, src)};
}

__device__ __forceinline__ df32 warp_sum_df(df32 x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = df_add(x, shfl_df(x, lane_id() ^ o));
  return x;
}

__device__ __forceinline__ double warp_sum_f64(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(kFull, x, o);
  return x;
}

}  // namespace lgbc
