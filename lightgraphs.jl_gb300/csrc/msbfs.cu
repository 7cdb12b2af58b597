// msbfs.cu -- multi-source (bit-lane) BFS with path counting and the
// reverse-level dependency sweep of Brandes' algorithm.
//
// Replaces, for up to 128 sources at once, the per-source loop body of
// betweenness_centrality (src/centrality/betweenness.jl:57-67):
//   forward  = dijkstra_shortest_paths(g, s; allpaths=true, trackvertices=true)
//              with unit weights (src/shortestpaths/dijkstra.jl:59-141): the
//              distance levels and the path counts sigma (:102,118)
//   backward = _accumulate_basic! (:81-107): delta[v] = sum over DAG
//              successors w of sigma[v] / sigma[w] * (1 + delta[w]), added to
//              betweenness[v] for v != s.
// Unit-weight Dijkstra visits vertices in BFS level order, and its
// predecessor lists are exactly the in-neighbours one level closer to the
// source, so a level-synchronous BFS reproduces sigma exactly (integers
// below 2^64 here; the reference's Float64 sums are exact below 2^53) and the
// dependencies up to summation order.
//
// Layout in HBM (per batch of <= 64 W sources, "lanes"; W = 1 or 2 64-bit
// words per lane set, a template parameter of every Brandes kernel):
//   visit[v]          W x uint64  lanes that reached v
//   mb[L & 1][v]      W x uint64  lanes for which v is at level L (dense)
//   sigma[v*64W + l]  uint64 path count (or FP64 in the overflow replay)
//   psi[v*64W + l]    df32 (1 + delta) / sigma (or FP64)
//   qv/qm             concatenated per-level lists of (vertex, lane set)
// A warp owns one vertex; thread t owns lanes 32 k + t (k < 2 W).  Edges are
// read 32 at a time; the edges that carry lanes are compacted in shared
// memory and walked edge by edge, each neighbour row read with coalesced
// loads.  Above the dense_edges tuning cut the warp instead transposes the
// 32 x 64W bit matrix (edge, lane) so that each thread walks only the edges
// on which its own lanes are set.  Hubs (more than hub_degree neighbours) are
// cut into kHubChunk-edge items processed by the whole grid (k_ms_hub_*).
// Stress, distance and level-statistics batches are one-word.
#include <algorithm>
#include <type_traits>

#include "lgbc_kernels.h"
#include "xf64.cuh"

namespace lgbc {
namespace {

__device__ __forceinline__ long long gwarp() {
  return (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
}
__device__ __forceinline__ long long nwarps() {
  return (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
}

// Level-parity buffer select (a runtime index into the by-value array would
// force the parameter struct into local memory).
__device__ __forceinline__ uint64_t* mb_at(const MsBuffers& b, int level) {
  return (level & 1) ? b.mb[1] : b.mb[0];
}

// ---------------------------------------------------------------------------
// Lane sets of a batch of 64 * W sources: W words per vertex, loaded and
// stored as one 8 * W-byte access.  Thread t of a warp owns the lanes
// 32 k + t, k < 2 W ("its lanes"); bit k of my_bits() and element k of the
// per-thread accumulator arrays below refer to lane 32 k + t.
// ---------------------------------------------------------------------------
template <int W> struct alignas(8 * W) Lanes {
  uint64_t w[W];
};

template <int W> __device__ __forceinline__ Lanes<W> lz() {
  Lanes<W> r;
#pragma unroll
  for (int j = 0; j < W; ++j) r.w[j] = 0ull;
  return r;
}
template <int W> __device__ __forceinline__ bool lany(const Lanes<W>& a) {
  uint64_t x = 0;
#pragma unroll
  for (int j = 0; j < W; ++j) x |= a.w[j];
  return x != 0ull;
}
template <int W> __device__ __forceinline__ Lanes<W> land(const Lanes<W>& a, const Lanes<W>& b) {
  Lanes<W> r;
#pragma unroll
  for (int j = 0; j < W; ++j) r.w[j] = a.w[j] & b.w[j];
  return r;
}
template <int W> __device__ __forceinline__ Lanes<W> lor(const Lanes<W>& a, const Lanes<W>& b) {
  Lanes<W> r;
#pragma unroll
  for (int j = 0; j < W; ++j) r.w[j] = a.w[j] | b.w[j];
  return r;
}
// a & ~b
template <int W> __device__ __forceinline__ Lanes<W> lminus(const Lanes<W>& a, const Lanes<W>& b) {
  Lanes<W> r;
#pragma unroll
  for (int j = 0; j < W; ++j) r.w[j] = a.w[j] & ~b.w[j];
  return r;
}
template <int W> __device__ __forceinline__ bool leq(const Lanes<W>& a, const Lanes<W>& b) {
  bool e = true;
#pragma unroll
  for (int j = 0; j < W; ++j) e = e && a.w[j] == b.w[j];
  return e;
}
template <int W> __device__ __forceinline__ Lanes<W> lshfl(const Lanes<W>& a, int src) {
  Lanes<W> r;
#pragma unroll
  for (int j = 0; j < W; ++j) r.w[j] = shfl_u64(a.w[j], src);
  return r;
}
template <int W> __device__ __forceinline__ Lanes<W> lwarp_or(const Lanes<W>& a) {
  Lanes<W> r;
#pragma unroll
  for (int j = 0; j < W; ++j) r.w[j] = warp_or_u64(a.w[j]);
  return r;
}
// The 32-bit half k (lanes 32 k .. 32 k + 31) of a lane set.
template <int W> __device__ __forceinline__ uint32_t lhalf(const Lanes<W>& a, int k) {
  return static_cast<uint32_t>(a.w[k >> 1] >> (32 * (k & 1)));
}
template <int W> __host__ __device__ __forceinline__ Lanes<W> lane_cast(const LaneSet& a) {
  Lanes<W> r;
#pragma unroll
  for (int j = 0; j < W; ++j) r.w[j] = a.w[j];
  return r;
}
template <int W> __device__ __forceinline__ Lanes<W>* lanes_of(uint64_t* p) {
  return reinterpret_cast<Lanes<W>*>(p);
}
template <int W> __device__ __forceinline__ const Lanes<W>* lanes_of(const uint64_t* p) {
  return reinterpret_cast<const Lanes<W>*>(p);
}
template <int W> __device__ __forceinline__ Lanes<W>* mbw(const MsBuffers& b, int level) {
  return lanes_of<W>(mb_at(b, level));
}
// The lanes present in the current frontier (BatchCtl::front_union).
template <int W> __device__ __forceinline__ Lanes<W> frontier_lanes(const BatchCtl* c) {
  Lanes<W> r;
#pragma unroll
  for (int j = 0; j < W; ++j) r.w[j] = c->front_union[j];
  return r;
}

template <int SK> struct Sig;
template <> struct Sig<kSigmaNone> {
  using T = unsigned long long;
  using Pair = ulonglong2;
};
template <> struct Sig<kSigmaU64> {
  using T = unsigned long long;
  using Pair = ulonglong2;
};
template <> struct Sig<kSigmaF64> {
  using T = double;
  using Pair = double2;
};
template <> struct Sig<kSigmaU64F64> {
  using T = unsigned long long;
  using Pair = ulonglong2;
};

// A path count as an FP64 value (uint64 counts round to nearest, as the
// reference's Float64 counts do above 2^53).
__device__ __forceinline__ double sigma_f64(unsigned long long x) { return __ull2double_rn(x); }
__device__ __forceinline__ double sigma_f64(double x) { return x; }

__device__ __forceinline__ void hub_add(unsigned long long* p, unsigned long long x) {
  atomicAdd(p, x);
}
__device__ __forceinline__ void hub_add(unsigned long long* p, double x) {
  atomicAdd(reinterpret_cast<double*>(p), x);
}

template <class T> __device__ __forceinline__ T from_bits(unsigned long long x);
template <> __device__ __forceinline__ unsigned long long from_bits(unsigned long long x) { return x; }
template <> __device__ __forceinline__ double from_bits(unsigned long long x) {
  return __longlong_as_double(static_cast<long long>(x));
}

// Bits (t, t + 32) of a one-word lane mask, as bit 0 / bit 1 (stress kernels).
__device__ __forceinline__ unsigned my_bits(uint64_t m) {
  const int ln = lane_id();
  return static_cast<unsigned>((m >> ln) & 1ull) |
         (static_cast<unsigned>((m >> (32 + ln)) & 1ull) << 1);
}

// Bit k = lane 32 k + t of a lane set, k < 2 W.
template <int W> __device__ __forceinline__ unsigned my_bits(const Lanes<W>& m) {
  const int ln = lane_id();
  unsigned r = 0;
#pragma unroll
  for (int k = 0; k < 2 * W; ++k) r |= ((lhalf(m, k) >> ln) & 1u) << k;
  return r;
}

__device__ __forceinline__ unsigned long long max_u64(unsigned long long a, unsigned long long b) {
  return a > b ? a : b;
}

// Store the path counts of this thread's lanes of w that are set in `mask`.
// Lanes outside `mask` may be read concurrently by other warps (w sits at
// another level for them), so they are never written.  Tracks the largest
// stored count (for the per-level overflow bound).
template <int SK, int W>
__device__ __forceinline__ void store_sigma(void* sigma, int32_t w, const Lanes<W>& mask,
                                            const typename Sig<SK>::T (&a)[2 * W],
                                            unsigned long long& smax) {
  using T = typename Sig<SK>::T;
  const int ln = lane_id();
  const unsigned my = my_bits(mask);
  T* row = reinterpret_cast<T*>(sigma) + static_cast<int64_t>(w) * (64 * W);
#pragma unroll
  for (int k = 0; k < 2 * W; ++k) {
    if (my & (1u << k)) {
      row[32 * k + ln] = a[k];
      if (SK == kSigmaU64) smax = max_u64(smax, static_cast<unsigned long long>(a[k]));
    }
  }
}

template <int W>
__device__ __forceinline__ void store_dist(int32_t* dist, int64_t ld, int32_t w, const Lanes<W>& mask,
                                           int32_t level) {
  const int ln = lane_id();
  const unsigned my = my_bits(mask);
#pragma unroll
  for (int k = 0; k < 2 * W; ++k)
    if (my & (1u << k)) dist[static_cast<int64_t>(32 * k + ln) * ld + w] = level;
}

// Compensated double-float accumulator: hi carries the running sum, lo the
// exact rounding errors of the hi additions plus the addends' own lo parts;
// normalised once at the end (acc_done).  The summed psi values are positive
// and so is the running sum, so the larger of the two hi operands is known
// by a max / min and Dekker's Fast2Sum gives the exact error of the hi
// addition (the same pair as Knuth's TwoSum) in 5 operations instead of 6.
__device__ __forceinline__ void acc_add(df32& acc, float xh, float xl) {
  const df32 t = fast_two_sum(fmaxf(acc.hi, xh), fminf(acc.hi, xh));
  acc.hi = t.hi;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(t.lo, xl));
}
__device__ __forceinline__ df32 acc_done(df32 acc) { return fast_two_sum(acc.hi, acc.lo); }

template <class T, class A> __device__ __forceinline__ void acc_row(A& acc, T x);
template <> __device__ __forceinline__ void acc_row(unsigned long long& acc, unsigned long long x) { acc += x; }
// FP64 dependencies: psi rows hold binary64 bits, summed by the gather
// accumulator (renormalised at the end of every 32-edge chunk).  In a
// two-word batch the first NF slots (lanes 0 .. 32 NF - 1) add on the FP64
// pipe instead (binary64 running sums, their bits kept in m) while the other
// slots add on the integer pipes: the two units work in parallel and neither
// carries all the adds.  NF is a property of the accumulator type, chosen per
// kernel from its measured FP64-pipe load.
template <int NF> struct XgAcc : xg64 {};

template <class A, int W> struct Fp64Slots {
  static constexpr int value = 0;
};
template <int NF, int W> struct Fp64Slots<XgAcc<NF>, W> {
  static constexpr int value = W == 1 ? 0 : NF * (W / 2);  // NF of every four slots
};

template <class T, class A, int W>
__device__ __forceinline__ void acc_slot(A& acc, T x, int k) {
  if constexpr (std::is_same<A, XgAcc<1>>::value || std::is_same<A, XgAcc<2>>::value) {
    if (k < Fp64Slots<A, W>::value)
      acc.m = static_cast<unsigned long long>(__double_as_longlong(
          __longlong_as_double(static_cast<long long>(acc.m)) +
          __longlong_as_double(static_cast<long long>(x))));
    else
      xg_add_bits(acc, x);
  } else {
    acc_row<T, A>(acc, x);
  }
}

template <class A> __device__ __forceinline__ void acc_chunk_end(A&) {}
template <int NF> __device__ __forceinline__ void acc_chunk_end(XgAcc<NF>& a) { xg_norm(a); }
template <int W, class A, int K> __device__ __forceinline__ void chunk_end(A (&a)[K]) {
#pragma unroll
  for (int k = 0; k < K; ++k)
    if (k >= Fp64Slots<A, W>::value) acc_chunk_end(a[k]);
}

// The extended value of slot k of a normalised gather accumulator.
template <int W, class A> __device__ __forceinline__ xf64 gather_value(const A& a, int k) {
  return k < Fp64Slots<A, W>::value ? xf_from_bits(a.m) : xg_to_xf(a);
}
template <> __device__ __forceinline__ void acc_row(double& acc, double x) { acc += x; }
template <> __device__ __forceinline__ void acc_row(df32& acc, float2 x) { acc_add(acc, x.x, x.y); }

template <class T> __device__ __forceinline__ T zero_row();
template <> __device__ __forceinline__ unsigned long long zero_row() { return 0ull; }
template <> __device__ __forceinline__ double zero_row() { return 0.0; }
template <> __device__ __forceinline__ float2 zero_row() { return make_float2(0.f, 0.f); }

template <class A> __device__ __forceinline__ A zero_acc();
template <> __device__ __forceinline__ unsigned long long zero_acc() { return 0ull; }
template <> __device__ __forceinline__ double zero_acc() { return 0.0; }
template <> __device__ __forceinline__ df32 zero_acc() { return df32{0.f, 0.f}; }
template <> __device__ __forceinline__ XgAcc<1> zero_acc() { return XgAcc<1>{}; }
template <> __device__ __forceinline__ XgAcc<2> zero_acc() { return XgAcc<2>{}; }

template <class A, int K> __device__ __forceinline__ void zero_accs(A (&a)[K]) {
#pragma unroll
  for (int k = 0; k < K; ++k) a[k] = zero_acc<A>();
}

// Per-warp staging of one chunk's contributing edges (compacted).
template <int W> struct ChunkStage {
  Lanes<W> f[kWarp];
  int32_t v[kWarp];
  int32_t j[kWarp];  // owner segment (seg_gather)
};
constexpr int kWarpsPerBlock = 8;  // every gather kernel runs 256-thread blocks

template <int W> __device__ __forceinline__ ChunkStage<W>& my_stage() {
  __shared__ ChunkStage<W> stage[kWarpsPerBlock];
  return stage[threadIdx.x >> 5];
}

// Rows gathered per step of a staged walk: 4 with one word, 2 with two (eight
// row loads in flight per thread either way).
template <int W> constexpr int kRowsInFlight = 4 / W;

// Chunk gather.  Each of the 32 threads holds one edge (neighbour id `nb`,
// lane set `f` of the lanes that edge contributes to).  Adds, for this
// thread's lanes 32 k + t, rows[nb_j * 64 W + 32 k + t] over every edge j whose
// set has that lane, into acc[k].
//  * at most `dense` contributing edges: the edges are compacted into shared
//    memory and the warp walks them, each edge's row read by coalesced loads;
//  * more: the (edge, lane) bit matrix is transposed so each thread walks only
//    the edges that carry its own lanes.
template <class T, class A, int W>
__device__ __forceinline__ void gather_chunk(int32_t nb, const Lanes<W>& f, const T* __restrict__ rows,
                                             int dense, A (&acc)[2 * W]) {
  constexpr int RS = 64 * W;
  constexpr int G = kRowsInFlight<W>;
  const int ln = lane_id();
  const unsigned bal = __ballot_sync(kFull, lany(f));
  if (bal == 0) return;
  const T* r0 = rows + ln;
  const int S = __popc(bal);
  if (S <= dense) {
    ChunkStage<W>& st = my_stage<W>();
    if (lany(f)) {
      const int r = __popc(bal & ((1u << ln) - 1u));
      st.v[r] = nb;
      st.f[r] = f;
    }
    __syncwarp();
    for (int r = 0; r < S; r += G) {
      T x[G][2 * W];
      unsigned my[G];
#pragma unroll
      for (int q = 0; q < G; ++q) {
        const bool ok = r + q < S;
        const Lanes<W> fj = ok ? st.f[r + q] : lz<W>();
        const int64_t off = static_cast<int64_t>(ok ? st.v[r + q] : 0) * RS;
        my[q] = my_bits(fj);
#pragma unroll
        for (int k = 0; k < 2 * W; ++k)  // x[q][k] is read below only under the same bit
          if (my[q] & (1u << k)) x[q][k] = r0[off + 32 * k];
      }
#pragma unroll
      for (int q = 0; q < G; ++q)
#pragma unroll
        for (int k = 0; k < 2 * W; ++k)
          if (my[q] & (1u << k)) acc_slot<T, A, W>(acc[k], x[q][k], k);
    }
    chunk_end<W>(acc);
    __syncwarp();
    return;
  }
  // transposed path: thread t gets the edges that carry its lane 32 k + t
  uint32_t E[2 * W];
#pragma unroll
  for (int k = 0; k < 2 * W; ++k) E[k] = warp_transpose32(lhalf(f, k));
#pragma unroll
  for (int k = 0; k < 2 * W; ++k) {
    const T* rb = r0 + 32 * k;
    uint32_t m = E[k];
    const int cnt = static_cast<int>(__reduce_max_sync(kFull, static_cast<unsigned>(__popc(m))));
    for (int c = 0; c < cnt; c += 4) {
      int32_t vj[4];
      bool ok[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        ok[q] = m != 0u;
        const int j = ok[q] ? __ffs(m) - 1 : 0;
        m &= m - 1u;
        vj[q] = __shfl_sync(kFull, nb, j);
      }
      T x[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        x[q] = zero_row<T>();
        if (ok[q]) x[q] = rb[static_cast<int64_t>(vj[q]) * RS];
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (ok[q]) acc_slot<T, A, W>(acc[k], x[q], k);
    }
  }
  chunk_end<W>(acc);
}

// Path-count gather over in-edges [e0, e1) of one vertex: for every
// in-neighbour v, f = front[v] & want marks the lanes whose predecessor it is;
// their rows are added into a.  Returns the union of all f (the lanes that
// discover the vertex).  With SK == kSigmaNone only the union is formed,
// and the scan stops once every wanted lane is found.
template <int SK, int W>
__device__ __forceinline__ Lanes<W> pull_range(const int32_t* __restrict__ ci, int64_t e0, int64_t e1,
                                               const Lanes<W>& want,
                                               const Lanes<W>* __restrict__ front,
                                               const void* __restrict__ sigma, int dense,
                                               typename Sig<SK>::T (&a)[2 * W]) {
  const int ln = lane_id();
  Lanes<W> found = lz<W>();
  if (SK == kSigmaNone) {
    for (int64_t e = e0; e < e1; e += kWarp) {
      const int64_t idx = e + ln;
      if (idx < e1) found = lor(found, land(front[ci[idx]], want));
      if (leq(lwarp_or(found), want)) break;
    }
    return lwarp_or(found);
  }
  // software-pipelined: the next chunk's neighbour ids and masks are loaded
  // before the current chunk's rows are gathered
  using T = typename Sig<SK>::T;
  int32_t v = 0;
  Lanes<W> f = lz<W>();
  if (e0 + ln < e1) {
    v = ci[e0 + ln];
    f = land(front[v], want);
  }
  for (int64_t e = e0; e < e1; e += kWarp) {
    const int64_t nidx = e + kWarp + ln;
    int32_t vn = 0;
    Lanes<W> fn = lz<W>();
    if (nidx < e1) {
      vn = ci[nidx];
      fn = land(front[vn], want);
    }
    found = lor(found, f);
    gather_chunk<T, T, W>(v, f, reinterpret_cast<const T*>(sigma), dense, a);
    v = vn;
    f = fn;
  }
  return lwarp_or(found);
}

// Dependency gather over out-edges [e0, e1) of v at level L: for every
// out-neighbour w, g = succ[w] & F marks the lanes for which w is a DAG
// successor; their psi = (1 + delta[w]) / sigma[w] are summed.
// (Software-pipelined like pull_range: the next chunk's ids and masks are in
// flight while the current chunk's rows are gathered.)  T / A: float2 / df32
// (df32 psi, normalised at the end) or double / double.
template <class T, class A, int W>
__device__ __forceinline__ void psi_range(const int32_t* __restrict__ ci, int64_t e0, int64_t e1,
                                          const Lanes<W>& F, const Lanes<W>* __restrict__ succ,
                                          const void* __restrict__ psi, int dense,
                                          A (&acc)[2 * W]) {
  const int ln = lane_id();
  int32_t w = 0;
  Lanes<W> gm = lz<W>();
  if (e0 + ln < e1) {
    w = ci[e0 + ln];
    gm = land(succ[w], F);
  }
  for (int64_t e = e0; e < e1; e += kWarp) {
    const int64_t nidx = e + kWarp + ln;
    int32_t wn = 0;
    Lanes<W> gn = lz<W>();
    if (nidx < e1) {
      wn = ci[nidx];
      gn = land(succ[wn], F);
    }
    gather_chunk<T, A, W>(w, gm, reinterpret_cast<const T*>(psi), dense, acc);
    w = wn;
    gm = gn;
  }
}

template <int W>
__device__ __forceinline__ void psi_range_df(const int32_t* __restrict__ ci, int64_t e0, int64_t e1,
                                             const Lanes<W>& F, const Lanes<W>* __restrict__ succ,
                                             const void* __restrict__ psi, int dense,
                                             df32 (&acc)[2 * W]) {
  psi_range<float2, df32, W>(ci, e0, e1, F, succ, psi, dense, acc);
#pragma unroll
  for (int k = 0; k < 2 * W; ++k) acc[k] = acc_done(acc[k]);
}

template <int W>
__device__ __forceinline__ void psi_range_f64(const int32_t* __restrict__ ci, int64_t e0, int64_t e1,
                                              const Lanes<W>& F, const Lanes<W>* __restrict__ succ,
                                              const void* __restrict__ psi, int dense,
                                              double (&acc)[2 * W]) {
  psi_range<double, double, W>(ci, e0, e1, F, succ, psi, dense, acc);
}

template <int W, int NF = 1>
__device__ __forceinline__ void psi_range_x(const int32_t* __restrict__ ci, int64_t e0, int64_t e1,
                                            const Lanes<W>& F, const Lanes<W>* __restrict__ succ,
                                            const void* __restrict__ psi, int dense,
                                            xf64 (&acc)[2 * W]) {
  XgAcc<NF> a[2 * W];
  zero_accs(a);
  psi_range<unsigned long long, XgAcc<NF>, W>(ci, e0, e1, F, succ, psi, dense, a);
#pragma unroll
  for (int k = 0; k < 2 * W; ++k) acc[k] = gather_value<W>(a[k], k);
}

__device__ __forceinline__ int64_t shfl_i64(int64_t x, int src) {
  return static_cast<int64_t>(shfl_u64(static_cast<uint64_t>(x), src));
}

// Segmented gather for low-degree graphs: lane j of the warp holds one
// vertex ("segment"): `valid`, its edge range [e0, e0 + deg) in `ci`, and a
// lane set `mask`.  The warp streams the concatenation of the valid
// segments' edges 32 at a time, so a vertex with a handful of edges does not
// occupy a whole warp pass; for an edge to neighbour x of segment j, the
// lanes f = gate[x] & mask_j contribute rows[x * 64 W + lane].  Contributing
// edges are compacted into shared memory with their segment, read a few at a
// time into per-thread accumulators acc[k] (lane 32 k + t); when the segment
// changes, flush(j, nm_j, acc) runs (warp-uniformly) with nm_j the union of
// segment j's f.  With VISIT_ALL every valid segment is flushed once,
// contributions or not.
template <class T, class A, bool VISIT_ALL, int W, class Flush>
__device__ __forceinline__ void seg_gather(bool valid, int64_t e0, int deg, const Lanes<W>& mask,
                                           const int32_t* __restrict__ ci,
                                           const Lanes<W>* __restrict__ gate,
                                           const T* __restrict__ rows, Flush&& flush) {
  constexpr int RS = 64 * W;
  constexpr int G = kRowsInFlight<W>;
  const int ln = lane_id();
  const int d = valid ? deg : 0;
  int incl = d;
#pragma unroll
  for (int o = 1; o < kWarp; o <<= 1) {
    const int y = __shfl_up_sync(kFull, incl, o);
    if (ln >= o) incl += y;
  }
  const int total = __shfl_sync(kFull, incl, kWarp - 1);
  const int off = incl - d;
  const unsigned vmask = __ballot_sync(kFull, valid);
  const T* r0 = rows + ln;
  ChunkStage<W>& st = my_stage<W>();
  int cur = -1;
  unsigned done = 0;
  Lanes<W> nm = lz<W>();
  A acc[2 * W];
  zero_accs(acc);
  for (int c = 0; c < total; c += kWarp) {
    const int gi = c + ln;
    int pos = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
      const int iv = __shfl_sync(kFull, incl, pos + step - 1);
      if (iv <= gi) pos += step;
    }
    const bool ok = gi < total;
    const int j = ok ? pos : 0;
    const int64_t ej = shfl_i64(e0, j);
    const int oj = __shfl_sync(kFull, off, j);
    const Lanes<W> mj = lshfl(mask, j);
    int32_t x = 0;
    Lanes<W> f = lz<W>();
    if (ok) {
      x = ci[ej + (gi - oj)];
      f = land(gate[x], mj);
    }
    const unsigned bal = __ballot_sync(kFull, lany(f));
    if (lany(f)) {
      const int r = __popc(bal & ((1u << ln) - 1u));
      st.v[r] = x;
      st.f[r] = f;
      st.j[r] = j;
    }
    __syncwarp();
    const int S = __popc(bal);
    for (int r = 0; r < S; r += G) {
      T xr[G][2 * W];
      unsigned my[G];
      Lanes<W> fq[G];
      int jq[G];
#pragma unroll
      for (int q = 0; q < G; ++q) {
        const bool okq = r + q < S;
        fq[q] = okq ? st.f[r + q] : lz<W>();
        jq[q] = okq ? st.j[r + q] : -1;
        const int64_t o = static_cast<int64_t>(okq ? st.v[r + q] : 0) * RS;
        my[q] = my_bits(fq[q]);
#pragma unroll
        for (int k = 0; k < 2 * W; ++k) {
          xr[q][k] = zero_row<T>();
          if (my[q] & (1u << k)) xr[q][k] = r0[o + 32 * k];
        }
      }
#pragma unroll
      for (int q = 0; q < G; ++q) {
        if (jq[q] < 0) continue;
        if (jq[q] != cur) {
          if (cur >= 0) {
            flush(cur, nm, acc);
            done |= 1u << cur;
          }
          cur = jq[q];
          nm = lz<W>();
          zero_accs(acc);
        }
        nm = lor(nm, fq[q]);
#pragma unroll
        for (int k = 0; k < 2 * W; ++k)
          if (my[q] & (1u << k)) acc_slot<T, A, W>(acc[k], xr[q][k], k);
      }
    }
    chunk_end<W>(acc);
    __syncwarp();
  }
  if (cur >= 0) {
    flush(cur, nm, acc);
    done |= 1u << cur;
  }
  if (VISIT_ALL) {
    unsigned rem = vmask & ~done;
    while (rem) {
      const int j = __ffs(rem) - 1;
      rem &= rem - 1;
      zero_accs(acc);
      flush(j, lz<W>(), acc);
    }
  }
}

// Finalise one lane l of v from its psi sum: delta = sigma * acc,
// psi[v] = (1 + delta) / sigma; returns delta.
__device__ __forceinline__ df32 finish_lane_df(const unsigned long long* srow, float2* prow, int l,
                                               df32 acc) {
  const df32 sv = df_from_u64(srow[l]);
  const df32 d = df_mul(sv, acc);
  const df32 p = df_div(df_add_f(d, 1.0f), sv);
  prow[l] = make_float2(p.hi, p.lo);
  return d;
}

// FP64 dependencies: delta = sigma * acc and psi = (1 + delta) / sigma in
// double, sigma read as uint64 (kSigmaU64F64) or double (kSigmaF64) counts.
template <class ST>
__device__ __forceinline__ double finish_lane_f64(const ST* srow, double* prow, int l, double acc) {
  const double sv = sigma_f64(srow[l]);
  const double d = sv * acc;
  prow[l] = (1.0 + d) / sv;
  return d;
}

// Finalise the dependencies of this thread's lanes `mine` (bit k = lane
// 32 k + t) of v from the psi sums; returns the lanes' delta sum.
template <int W>
__device__ __forceinline__ df32 finish_df(void* psi, const void* sigma, int32_t v, unsigned mine,
                                          const df32 (&acc)[2 * W]) {
  const int ln = lane_id();
  df32 contrib{0.f, 0.f};
  if (!mine) return contrib;
  const unsigned long long* srow =
      reinterpret_cast<const unsigned long long*>(sigma) + static_cast<int64_t>(v) * (64 * W);
  float2* prow = reinterpret_cast<float2*>(psi) + static_cast<int64_t>(v) * (64 * W);
  if (mine & 1u) contrib = finish_lane_df(srow, prow, ln, acc[0]);
#pragma unroll
  for (int k = 1; k < 2 * W; ++k)
    if (mine & (1u << k)) contrib = df_add(contrib, finish_lane_df(srow, prow, 32 * k + ln, acc[k]));
  return contrib;
}

template <int SK, int W>
__device__ __forceinline__ double finish_f64(void* psi, const void* sigma, int32_t v, unsigned mine,
                                             const double (&acc)[2 * W]) {
  using ST = typename Sig<SK>::T;
  const int ln = lane_id();
  double contrib = 0.0;
  if (!mine) return contrib;
  const ST* srow = reinterpret_cast<const ST*>(sigma) + static_cast<int64_t>(v) * (64 * W);
  double* prow = reinterpret_cast<double*>(psi) + static_cast<int64_t>(v) * (64 * W);
#pragma unroll
  for (int k = 0; k < 2 * W; ++k)
    if (mine & (1u << k)) contrib += finish_lane_f64(srow, prow, 32 * k + ln, acc[k]);
  return contrib;
}

// FP64 dependencies from an extended psi sum (kSigmaU64F64): with acc =
// sum of the successors' psi = delta / sigma, psi = 1 / sigma + acc (the
// reference's coeff, (1 + delta) / sigma) is stored as binary64 and
// delta = sigma * acc is returned; the path count stays an exact integer.
__device__ __forceinline__ xf64 finish_lane_x(const unsigned long long* srow,
                                              unsigned long long* prow, int l, xf64 acc) {
  const unsigned long long sv = srow[l];
  prow[l] = xf_to_bits(xf_add(acc, xf_recip_u64(sv)));
  return xf_mul_u64(acc, sv);
}

// Finalise this thread's lanes `mine` of v; returns the sum of their deltas
// (lw: per-lane weights, or null).
template <int W>
__device__ __forceinline__ xf64 finish_x(void* psi, const void* sigma, int32_t v, unsigned mine,
                                         const xf64 (&acc)[2 * W], const double* __restrict__ lw) {
  const int ln = lane_id();
  xf64 contrib = xf_zero();
  if (!mine) return contrib;
  const unsigned long long* srow =
      reinterpret_cast<const unsigned long long*>(sigma) + static_cast<int64_t>(v) * (64 * W);
  unsigned long long* prow = reinterpret_cast<unsigned long long*>(psi) + static_cast<int64_t>(v) * (64 * W);
#pragma unroll
  for (int k = 0; k < 2 * W; ++k)
    if (mine & (1u << k)) {
      xf64 d = finish_lane_x(srow, prow, 32 * k + ln, acc[k]);
      if (lw) d = xf_mul(d, xf_from_bits(__double_as_longlong(lw[32 * k + ln])));
      contrib = xf_add(contrib, d);
    }
  return contrib;
}

// Sum over the warp (zeros allowed): every value is aligned to the largest
// exponent and the 63-bit significands are added exactly as four 16-bit
// pieces by redux (each piece sum < 2^21); the total (< 2^68) keeps its top
// 63 bits.  Relative error < 2^-56.
__device__ __forceinline__ xf64 warp_sum_x(xf64 a) {
  const int E = static_cast<int>(__reduce_max_sync(kFull, static_cast<unsigned>(a.e)));
  if (E == 0) return xf_zero();  // every value is zero (warp-uniform)
  const uint64_t m = xf_shr(a.m, static_cast<uint32_t>(E - a.e));
  const uint32_t lo = static_cast<uint32_t>(m), hi = static_cast<uint32_t>(m >> 32);
  const uint64_t s0 = __reduce_add_sync(kFull, lo & 0xFFFFu);
  const uint64_t s1 = __reduce_add_sync(kFull, lo >> 16);
  const uint64_t s2 = __reduce_add_sync(kFull, hi & 0xFFFFu);
  const uint64_t s3 = __reduce_add_sync(kFull, hi >> 16);
  // total >> 5 = s3 2^43 + s2 2^27 + s1 2^11 + s0 2^-5 < 2^63
  const uint64_t t = (s3 << 43) + (s2 << 27) + (s1 << 11) + (s0 >> 5);
  const int lz = xf_clz(t) - 1;  // 0..5: the largest value alone is >= 2^57 after the shift
  return xf64{t << lz, E + 5 - lz};
}

// bc[v] += x, rounded once (lane 0 of the warp that owns v at this level).
__device__ __forceinline__ void bc_add_x(double* bc, int32_t v, xf64 x) {
  if (x.m == 0) return;
  unsigned long long* p = reinterpret_cast<unsigned long long*>(bc) + v;
  *p = xf_to_bits(xf_add_bits(x, *p));
}

// The lane weights of vertex v (its copy's row in a stacked union; stacked
// unions are one-word batches).
template <int W> __device__ __forceinline__ const double* weights_of(const MsBuffers& b, int32_t v) {
  return b.lane_w_n > 0 ? b.lane_w + (static_cast<int64_t>(v) / b.lane_w_n) * (64 * W) : b.lane_w;
}

// Weighted finalisation (importance-sampled estimators): the same psi
// updates, returning sum over the lanes of w[lane] * delta in FP64.
template <int W>
__device__ __forceinline__ double finish_df_w(void* psi, const void* sigma, int32_t v,
                                              unsigned mine, const df32 (&acc)[2 * W],
                                              const double* __restrict__ lw) {
  const int ln = lane_id();
  double contrib = 0.0;
  if (!mine) return contrib;
  const unsigned long long* srow =
      reinterpret_cast<const unsigned long long*>(sigma) + static_cast<int64_t>(v) * (64 * W);
  float2* prow = reinterpret_cast<float2*>(psi) + static_cast<int64_t>(v) * (64 * W);
#pragma unroll
  for (int k = 0; k < 2 * W; ++k)
    if (mine & (1u << k))
      contrib += lw[32 * k + ln] * df_to_double(finish_lane_df(srow, prow, 32 * k + ln, acc[k]));
  return contrib;
}

template <int SK, int W>
__device__ __forceinline__ double finish_f64_w(void* psi, const void* sigma, int32_t v,
                                               unsigned mine, const double (&acc)[2 * W],
                                               const double* __restrict__ lw) {
  using ST = typename Sig<SK>::T;
  const int ln = lane_id();
  double contrib = 0.0;
  if (!mine) return contrib;
  const ST* srow = reinterpret_cast<const ST*>(sigma) + static_cast<int64_t>(v) * (64 * W);
  double* prow = reinterpret_cast<double*>(psi) + static_cast<int64_t>(v) * (64 * W);
#pragma unroll
  for (int k = 0; k < 2 * W; ++k)
    if (mine & (1u << k)) contrib += lw[32 * k + ln] * finish_lane_f64(srow, prow, 32 * k + ln, acc[k]);
  return contrib;
}

__device__ __forceinline__ df32 df_from_double(double x) {
  const float hi = __double2float_rn(x);
  const float lo = __double2float_rn(x - static_cast<double>(hi));
  return df32{hi, lo};
}

// Last-item handshake of a hub: fence this item's atomics, count it, and
// report (warp-uniformly) whether it was the hub's last item.
__device__ __forceinline__ bool hub_last(unsigned int* cnt, int nitems) {
  __threadfence();
  unsigned last = 0;
  if (lane_id() == 0) last = atomicAdd(cnt, 1u) == static_cast<unsigned>(nitems - 1) ? 1u : 0u;
  last = __shfl_sync(kFull, last, 0);
  if (last) __threadfence();
  return last != 0;
}

// ---------------------------------------------------------------------------
// Batch initialisation: level 0 = the sources (one lane each; a repeated
// source gets several lanes in one list entry).  One block, thread l = lane
// l: the lanes OR themselves into their source's lane set, and the first lane
// of each distinct source appends it, in lane order (its position is the
// number of first lanes before it).
// ---------------------------------------------------------------------------
template <int SK, int W>
__global__ void __launch_bounds__(kWideLanes) k_ms_init(DevGraph g, MsBuffers b, int nl, Lanes<W> act,
                                                        unsigned long long cap,
                                                        unsigned long long sigma_limit,
                                                        int32_t* dist, int64_t ld) {
  using T = typename Sig<SK>::T;
  __shared__ int32_t src[kWideLanes];
  __shared__ unsigned firsts[kWideLanes / kWarp];
  __shared__ unsigned long long sums[2];  // out-degrees of the sources, in-degrees of finished ones
  Lanes<W>* front = lanes_of<W>(b.mb[0]);
  Lanes<W>* qm = lanes_of<W>(b.qm);
  Lanes<W>* visit = lanes_of<W>(b.visit);
  const int l = static_cast<int>(threadIdx.x);
  const bool live = l < nl;
  const int32_t s = live ? b.lane_src[l] : -1;
  src[l] = s;
  if (l < 2) sums[l] = 0ull;
  __syncthreads();
  if (live) {
    atomicOr(reinterpret_cast<unsigned long long*>(&front[s].w[l >> 6]), 1ull << (l & 63));
    if (SK != kSigmaNone) reinterpret_cast<T*>(b.sigma)[static_cast<int64_t>(s) * (64 * W) + l] = T(1);
    if (dist) dist[static_cast<int64_t>(l) * ld + s] = 0;
  }
  bool first = live;
  for (int j = 0; j < l && first; ++j) first = src[j] != s;
  const unsigned bal = __ballot_sync(kFull, first);
  if (lane_id() == 0) firsts[l >> 5] = static_cast<unsigned>(__popc(bal));
  __syncthreads();  // also completes every lane's OR before the lane sets are read
  unsigned pos = static_cast<unsigned>(__popc(bal & ((1u << lane_id()) - 1u)));
  unsigned total = 0;
  for (int wi = 0; wi < kWideLanes / kWarp; ++wi) {
    if (wi < (l >> 5)) pos += firsts[wi];
    total += firsts[wi];
  }
  if (first) {
    const Lanes<W> m = front[s];
    b.qv[pos] = s;
    qm[pos] = m;
    visit[s] = m;
    atomicAdd(&sums[0], static_cast<unsigned long long>(g.rowptr[s + 1] - g.rowptr[s]));
    if (leq(m, act))
      atomicAdd(&sums[1], static_cast<unsigned long long>(g.in_rowptr[s + 1] - g.in_rowptr[s]));
  }
  __syncthreads();
  if (l != 0) return;
  BatchCtl* c = b.ctl;
  c->lo = 0;
  c->hi = total;
  c->tail = total;
  c->mf = 0;
  c->mf_cur = sums[0];
  c->mu_done = sums[1];
  c->cap = cap;
  c->level = 0;
  c->maxlevel = 0;
  c->done = 0;
  c->overflow_list = 0;
  c->overflow_sigma = 0;
  c->mode = 0;
  c->sigma_max = 1;
  c->sigma_limit = sigma_limit;
  c->td_levels = 0;
  c->bu_levels = 0;
  c->runaway = 0;
  for (int j = 0; j < kMaxWords; ++j) {
    c->front_union[j] = j < W ? act.w[j % W] : 0ull;
    c->next_union[j] = 0ull;
  }
  b.lvl_off[0] = 0;
  b.lvl_off[1] = total;
}

// ---------------------------------------------------------------------------
// Top-down, phase 1: expand Q_L over out-edges; the first lane set on a new
// vertex appends it to Q_{L+1}.  next[w] collects the discovering lanes.
// With two words the words are ORed separately, so the first discoverer is
// decided by a per-vertex claim flag instead (cleared by the settle phase).
// ---------------------------------------------------------------------------
template <int W>
__device__ __forceinline__ void discover_range(const int32_t* __restrict__ ci, int64_t e0, int64_t e1,
                                               const Lanes<W>& F, const Lanes<W>* __restrict__ visit,
                                               Lanes<W>* next, unsigned* claim, int32_t* qv,
                                               BatchCtl* c) {
  const int ln = lane_id();
  for (int64_t e = e0; e < e1; e += kWarp) {
    const int64_t idx = e + ln;
    bool app = false;
    int32_t w = 0;
    if (idx < e1) {
      w = ci[idx];
      const Lanes<W> m = lminus(F, visit[w]);
      if (lany(m)) {
        unsigned long long* nw = reinterpret_cast<unsigned long long*>(next[w].w);
        if (W == 1) {
          app = atomicOr(nw, m.w[0]) == 0ull;
        } else {
#pragma unroll
          for (int j = 0; j < W; ++j)
            if (m.w[j]) atomicOr(nw + j, m.w[j]);
          app = atomicExch(claim + w, 1u) == 0u;
        }
      }
    }
    const unsigned long long slot = warp_append(app, &c->tail);
    if (app) qv[slot] = w;
  }
}

template <int W>
__global__ void __launch_bounds__(256) k_ms_td_discover(DevGraph g, MsBuffers b, HubData hd) {
  BatchCtl* c = b.ctl;
  const unsigned long long lo = c->lo, hi = c->hi;
  const int L = c->level;
  Lanes<W>* next = mbw<W>(b, L + 1);
  const Lanes<W>* qm = lanes_of<W>(b.qm);
  const Lanes<W>* visit = lanes_of<W>(b.visit);
  for (unsigned long long i = lo + gwarp(); i < hi; i += nwarps()) {
    const int32_t v = b.qv[i];
    const int64_t e0 = g.rowptr[v], e1 = g.rowptr[v + 1];
    if (e1 - e0 > hd.hub_degree) continue;  // k_ms_hub_discover
    discover_range<W>(g.colidx, e0, e1, qm[i], visit, next, b.claim, b.qv, c);
  }
}

template <int W>
__global__ void __launch_bounds__(256) k_ms_hub_discover(DevGraph g, MsBuffers b, HubData hd) {
  BatchCtl* c = b.ctl;
  const int L = c->level;
  const Lanes<W>* front = mbw<W>(b, L);
  Lanes<W>* next = mbw<W>(b, L + 1);
  const Lanes<W>* visit = lanes_of<W>(b.visit);
  for (long long it = gwarp(); it < hd.n_out; it += nwarps()) {
    const HubItem I = hd.out_items[it];
    const Lanes<W> F = front[I.v];
    if (!lany(F)) continue;
    discover_range<W>(g.colidx, I.lo, I.hi, F, visit, next, b.claim, b.qv, c);
  }
}

// Top-down, phase 2: for every vertex appended in phase 1, record its lane
// set, mark it visited and pull its path counts from its predecessors
// (hubs: k_ms_hub_pull).
template <int SK, bool DIST, int W>
__global__ void __launch_bounds__(256, W == 4 ? 3 : 4) k_ms_td_settle(DevGraph g, MsBuffers b, HubData hd,
                                                      Lanes<W> act, int32_t* dist, int64_t ld) {
  using T = typename Sig<SK>::T;
  BatchCtl* c = b.ctl;
  const unsigned long long lo = c->hi, hi = c->tail;
  const int L = c->level;
  const Lanes<W>* __restrict__ front = mbw<W>(b, L);
  const Lanes<W>* __restrict__ next = mbw<W>(b, L + 1);
  Lanes<W>* qm = lanes_of<W>(b.qm);
  Lanes<W>* visit = lanes_of<W>(b.visit);
  const int ln = lane_id();
  unsigned long long mf = 0, mu = 0, smax = 0;
  for (unsigned long long i = lo + gwarp(); i < hi; i += nwarps()) {
    const int32_t w = b.qv[i];
    const Lanes<W> mask = next[w];
    const int64_t e0 = g.in_rowptr[w], e1 = g.in_rowptr[w + 1];
    if (ln == 0) {
      const Lanes<W> nv = lor(visit[w], mask);
      qm[i] = mask;
      visit[w] = nv;
      if (W > 1) b.claim[w] = 0u;
      mf += static_cast<unsigned long long>(g.rowptr[w + 1] - g.rowptr[w]);
      if (leq(nv, act)) mu += static_cast<unsigned long long>(e1 - e0);
    }
    if (DIST) store_dist(dist, ld, w, mask, L + 1);
    if (SK != kSigmaNone && e1 - e0 <= hd.hub_degree) {
      T a[2 * W];
      zero_accs(a);
      pull_range<SK, W>(g.in_colidx, e0, e1, mask, front, b.sigma, hd.dense_edges, a);
      store_sigma<SK, W>(b.sigma, w, mask, a, smax);
    }
  }
  if (SK == kSigmaU64) {
    smax = warp_max_u64(smax);
    if (ln == 0 && smax) atomicMax(&c->sigma_max, smax);
  }
  if (ln == 0) {
    if (mf) atomicAdd(&c->mf, mf);
    if (mu) atomicAdd(&c->mu_done, mu);
  }
}

// ---------------------------------------------------------------------------
// Bottom-up: every vertex some lane has not reached scans its in-neighbours
// for predecessors in the current frontier.  A warp takes 32 consecutive
// vertices, so its discoveries are appended with one atomic.  Hubs are left
// to k_ms_hub_pull.
// ---------------------------------------------------------------------------
template <int SK, bool DIST, int W, bool LF>
__global__ void __launch_bounds__(256, W == 4 ? 3 : 4) k_ms_bu(DevGraph g, MsBuffers b, HubData hd, Lanes<W> act,
                                               int32_t* dist, int64_t ld) {
  using T = typename Sig<SK>::T;
  BatchCtl* c = b.ctl;
  const int L = c->level;
  const Lanes<W>* __restrict__ front = mbw<W>(b, L);
  Lanes<W>* next = mbw<W>(b, L + 1);
  Lanes<W>* qm = lanes_of<W>(b.qm);
  Lanes<W>* visit = lanes_of<W>(b.visit);
  const int64_t n = g.n;
  const int ln = lane_id();
  unsigned long long mf = 0, mu = 0, smax = 0;
  // the lanes each of the warp's 32 vertices discovers, kept in shared memory
  // rather than in registers across the candidate loop; with LF the lanes of
  // the frontier are read once per block and bound the wanted lanes
  __shared__ Lanes<W> found_of[kWarpsPerBlock][kWarp];
  __shared__ Lanes<W> live;
  Lanes<W>* my_found = found_of[threadIdx.x >> 5];
  if (LF) {
    if (threadIdx.x == 0) live = frontier_lanes<W>(c);
    __syncthreads();
  }
  for (int64_t base = gwarp() * kWarp; base < n; base += nwarps() * kWarp) {
    const int64_t wme = base + ln;
    bool cand = false;
    my_found[ln] = lz<W>();
    if (wme < n) {
      const int64_t d = g.in_rowptr[wme + 1] - g.in_rowptr[wme];
      cand = (LF ? lany(land(lminus(act, visit[wme]), live)) : !leq(visit[wme], act)) && d > 0 &&
             d <= hd.hub_degree;
    }
    unsigned cb = __ballot_sync(kFull, cand);
    __syncwarp();
    while (cb) {
      const int j = __ffs(cb) - 1;
      cb &= cb - 1;
      const int32_t w = static_cast<int32_t>(base + j);
      const Lanes<W> want = LF ? land(lminus(act, visit[w]), live) : lminus(act, visit[w]);
      T a[2 * W];
      zero_accs(a);
      const Lanes<W> nm = pull_range<SK, W>(g.in_colidx, g.in_rowptr[w], g.in_rowptr[w + 1], want,
                                            front, b.sigma, hd.dense_edges, a);
      if (lany(nm)) {
        if (SK != kSigmaNone) store_sigma<SK, W>(b.sigma, w, nm, a, smax);
        if (DIST) store_dist(dist, ld, w, nm, L + 1);
      }
      if (ln == j) my_found[j] = nm;
    }
    __syncwarp();
    const Lanes<W> my_nm = my_found[ln];
    const bool app = lany(my_nm);
    const unsigned long long slot = warp_append(app, &c->tail);
    if (app) {
      b.qv[slot] = static_cast<int32_t>(wme);
      qm[slot] = my_nm;
      next[wme] = my_nm;
      const Lanes<W> nv = lor(visit[wme], my_nm);
      visit[wme] = nv;
      mf += static_cast<unsigned long long>(g.rowptr[wme + 1] - g.rowptr[wme]);
      if (leq(nv, act)) mu += static_cast<unsigned long long>(g.in_rowptr[wme + 1] - g.in_rowptr[wme]);
    }
  }
  if (SK == kSigmaU64) {
    smax = warp_max_u64(smax);
    if (ln == 0 && smax) atomicMax(&c->sigma_max, smax);
  }
  mf = warp_sum_u64(mf);
  mu = warp_sum_u64(mu);
  if (ln == 0) {
    if (mf) atomicAdd(&c->mf, mf);
    if (mu) atomicAdd(&c->mu_done, mu);
  }
}

// Hub path-count pull over in-edge items, for the top-down settle phase
// (BU == false: the hub was discovered this level, want = next[h]) or the
// bottom-up phase (BU == true: the hub is not finished, want = unvisited
// lanes).  Partial sums go to the hub's slot; its last item stores sigma and,
// bottom-up, appends the hub to the next level.
template <int SK, bool DIST, bool BU, int W, bool LF>
__global__ void __launch_bounds__(256, W == 4 ? 3 : 4) k_ms_hub_pull(DevGraph g, MsBuffers b, HubData hd,
                                                     Lanes<W> act, int32_t* dist, int64_t ld) {
  using T = typename Sig<SK>::T;
  BatchCtl* c = b.ctl;
  const int L = c->level;
  const Lanes<W>* __restrict__ front = mbw<W>(b, L);
  Lanes<W>* next = mbw<W>(b, L + 1);
  Lanes<W>* qm = lanes_of<W>(b.qm);
  Lanes<W>* visit = lanes_of<W>(b.visit);
  const int ln = lane_id();
  unsigned long long mf = 0, mu = 0, smax = 0;
  for (long long it = gwarp(); it < hd.n_in; it += nwarps()) {
    const HubItem I = hd.in_items[it];
    const int32_t h = I.v;
    Lanes<W> vis = lz<W>(), want;
    if (BU) {
      // every item of a hub reads the same visit[h] and frontier lanes, so
      // all of them skip it or none does (the last-item count stays whole)
      vis = visit[h];
      want = lminus(act, vis);
      if (LF) want = land(want, frontier_lanes<W>(c));
      if (!lany(want)) continue;
    } else {
      want = next[h];
      if (!lany(want)) continue;
    }
    T a[2 * W];
    zero_accs(a);
    const Lanes<W> found =
        pull_range<SK, W>(g.in_colidx, I.lo, I.hi, want, front, b.sigma, hd.dense_edges, a);
    unsigned long long* acc = hd.acc + static_cast<int64_t>(I.slot) * (64 * W);
    unsigned long long* hmask = hd.mask + static_cast<int64_t>(I.slot) * W;
    if (SK != kSigmaNone) {
#pragma unroll
      for (int k = 0; k < 2 * W; ++k)
        if (a[k] != T(0)) hub_add(acc + 32 * k + ln, a[k]);
    }
    if (BU && ln == 0) {
#pragma unroll
      for (int j = 0; j < W; ++j)
        if (found.w[j]) atomicOr(hmask + j, found.w[j]);
    }
    if (!hub_last(hd.cnt + I.slot, I.nitems)) continue;
    Lanes<W> nm = want;
    if (BU) {
#pragma unroll
      for (int j = 0; j < W; ++j) {
        unsigned long long x = 0;
        if (ln == 0) x = atomicExch(hmask + j, 0ull);
        nm.w[j] = shfl_u64(x, 0);
      }
    }
    T s[2 * W];
#pragma unroll
    for (int k = 0; k < 2 * W; ++k) {
      s[k] = T(0);
      if (SK != kSigmaNone) s[k] = from_bits<T>(atomicExch(acc + 32 * k + ln, 0ull));
    }
    if (ln == 0) hd.cnt[I.slot] = 0u;
    if (lany(nm)) {
      if (SK != kSigmaNone) store_sigma<SK, W>(b.sigma, h, nm, s, smax);
      if (DIST) store_dist(dist, ld, h, nm, L + 1);
      if (BU && ln == 0) {
        const unsigned long long slot = atomicAdd(&c->tail, 1ull);
        b.qv[slot] = h;
        qm[slot] = nm;
        next[h] = nm;
        const Lanes<W> nv = lor(vis, nm);
        visit[h] = nv;
        mf += static_cast<unsigned long long>(g.rowptr[h + 1] - g.rowptr[h]);
        if (leq(nv, act)) mu += static_cast<unsigned long long>(g.in_rowptr[h + 1] - g.in_rowptr[h]);
      }
    }
  }
  if (SK == kSigmaU64) {
    smax = warp_max_u64(smax);
    if (ln == 0 && smax) atomicMax(&c->sigma_max, smax);
  }
  if (ln == 0) {
    if (mf) atomicAdd(&c->mf, mf);
    if (mu) atomicAdd(&c->mu_done, mu);
  }
}

// After a level: clear the old frontier's dense masks (kept when the forward
// sweep just ended, because the backward sweep starts from them).
// With LF (digraphs) it also ORs the lane sets of the new level Q_{L+1} =
// list[hi, tail) into ctl->next_union (per block in shared memory, then only
// the bits not yet set), the frontier lanes of the next bottom-up level.
template <int W, bool LF>
__global__ void k_ms_clear_front(MsBuffers b) {
  __shared__ unsigned long long blk[W];
  BatchCtl* c = b.ctl;
  if (c->tail == c->hi) return;  // uniform: the sweep ended
  const unsigned long long lo = c->lo, hi = c->hi, tail = c->tail;
  Lanes<W>* front = mbw<W>(b, c->level);
  const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
  for (unsigned long long i = lo + blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += stride)
    front[b.qv[i]] = lz<W>();
  if (!LF) return;
  if (threadIdx.x < W) blk[threadIdx.x] = 0ull;
  __syncthreads();
  const Lanes<W>* qm = lanes_of<W>(b.qm);
  Lanes<W> u = lz<W>();
  for (unsigned long long i = hi + blockIdx.x * blockDim.x + threadIdx.x; i < tail; i += stride)
    u = lor(u, qm[i]);
  u = lwarp_or(u);
  if (lane_id() == 0) {
#pragma unroll
    for (int j = 0; j < W; ++j)
      if (u.w[j]) atomicOr(&blk[j], u.w[j]);
  }
  __syncthreads();
  if (threadIdx.x < W) {
    const unsigned long long mine = blk[threadIdx.x];
    const unsigned long long have = *reinterpret_cast<volatile unsigned long long*>(&c->next_union[threadIdx.x]);
    if (mine & ~have) atomicOr(&c->next_union[threadIdx.x], mine);
  }
}

__device__ __forceinline__ void advance_step(const MsBuffers& b, int64_t n);

__global__ void k_ms_advance(MsBuffers b, int64_t n) { advance_step(b, n); }

// Device-driven level loops (CUDA graphs with conditional nodes).  The
// forward loop is WHILE(loop) { SWITCH(dir) { 0: top-down level, 1:
// bottom-up level }; k_loop_advance }; the backward loop is WHILE(loop) {
// dependency level; k_loop_back_advance }.  Handles default to 0 (stop) and
// are set only by these single-thread kernels; every forward iteration either
// raises the level or ends the loop, and the level is capped at lp.max_levels,
// so both loops are bounded.
// (The direction handle belongs to the loop body and starts every launch at 0:
// the first level is expanded top-down.)
__global__ void k_loop_arm(MsBuffers b, LoopParams lp) {
  const BatchCtl* c = b.ctl;
  cudaGraphSetConditional(lp.loop, c->done == 0 ? 1u : 0u);
}

__global__ void k_loop_advance(MsBuffers b, LoopParams lp) {
  BatchCtl* c = b.ctl;
  if (c->mode) c->bu_levels += 1; else c->td_levels += 1;
  advance_step(b, lp.n);
  bool stop = c->done || c->overflow_list || (u64_counts(lp.sigma_kind) && c->overflow_sigma);
  if (!stop && c->level >= lp.max_levels) {
    c->runaway = 1;
    stop = true;
  }
  unsigned dir = 2u;
  if (!stop) {
    // Beamer's switch on the union of the lanes, as the host-driven loop does
    const double mf = static_cast<double>(c->mf_cur);
    const double mu = static_cast<double>(lp.nnz) - static_cast<double>(c->mu_done);
    const double nf = static_cast<double>(c->hi - c->lo);
    const bool bu = c->mode ? (nf >= static_cast<double>(lp.n) / lp.beta) : (mf > mu / lp.alpha);
    c->mode = bu ? 1 : 0;
    dir = bu ? 1u : 0u;
  }
  cudaGraphSetConditional(lp.loop, stop ? 0u : 1u);
  cudaGraphSetConditional(lp.dir, dir);
}

__global__ void k_loop_back_arm(MsBuffers b, LoopParams lp) {
  BatchCtl* c = b.ctl;
  c->level = c->maxlevel;
  cudaGraphSetConditional(lp.loop, c->maxlevel >= 0 ? 1u : 0u);
}

__global__ void k_loop_back_advance(MsBuffers b, LoopParams lp) {
  BatchCtl* c = b.ctl;
  c->level -= 1;
  cudaGraphSetConditional(lp.loop, c->level >= 0 ? 1u : 0u);
}

__device__ __forceinline__ void advance_step(const MsBuffers& b, int64_t n) {
  BatchCtl* c = b.ctl;
  const int L = c->level;
  b.lvl_off[L + 2] = c->tail;
  // every count of level L + 1 is a sum of at most max-in-degree counts of
  // level L; once a level's largest count passes the limit, the next level
  // could overflow 64 bits, so the batch is replayed with FP64 counts
  if (c->sigma_max > c->sigma_limit) c->overflow_sigma = 1;
  c->sigma_max = 0;
  if (c->tail == c->hi) {
    c->done = 1;
    c->maxlevel = L;
    c->mf_cur = 0;
    return;
  }
  c->lo = c->hi;
  c->hi = c->tail;
  c->level = L + 1;
  c->mf_cur = c->mf;
  c->mf = 0;
  for (int j = 0; j < kMaxWords; ++j) {
    c->front_union[j] = c->next_union[j];
    c->next_union[j] = 0ull;
  }
  if (c->cap - c->tail < static_cast<unsigned long long>(n)) c->overflow_list = 1;
}

__global__ void k_ms_begin_backward(MsBuffers b) { b.ctl->level = b.ctl->maxlevel; }

// Backward step at level L, part 1: mb[L & 1] still holds F_{L+2}; clear it.
template <int W>
__global__ void k_ms_back_clear(MsBuffers b) {
  BatchCtl* c = b.ctl;
  const int L = c->level;
  if (L + 2 > c->maxlevel) return;
  const unsigned long long lo = b.lvl_off[L + 2], hi = b.lvl_off[L + 3];
  Lanes<W>* other = mbw<W>(b, L);
  for (unsigned long long i = lo + blockIdx.x * blockDim.x + threadIdx.x; i < hi;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x)
    other[b.qv[i]] = lz<W>();
}

// Backward step at level L, part 2 (pull): for every (v, lane) at level L,
//   delta = sigma[v] * sum_{w in out(v), lane at level L+1 of w} psi[w]
//   psi[v] = (1 + delta) / sigma[v]
// and betweenness[v] += sum over lanes of delta (level 0 = sources: skipped,
// as _accumulate_basic! skips w == s, betweenness.jl:102).
// psi is the reference's `coeff` (betweenness.jl:96) stored once per vertex.
// Writes F_L into mb[L & 1] for every v (hubs included) before
// k_ms_hub_delta finishes the hubs.
template <int SK, int W>
__global__ void __launch_bounds__(256, W == 1 ? 5 : (W == 2 ? 4 : 3)) k_ms_delta(DevGraph g, MsBuffers b, HubData hd, double* bc) {
  BatchCtl* c = b.ctl;
  const int L = c->level;
  const unsigned long long lo = b.lvl_off[L], hi = b.lvl_off[L + 1];
  const Lanes<W>* __restrict__ succ = mbw<W>(b, L + 1);
  Lanes<W>* other = mbw<W>(b, L);
  const Lanes<W>* qm = lanes_of<W>(b.qm);
  Lanes<W>* visit = lanes_of<W>(b.visit);
  const int ln = lane_id();
  for (unsigned long long i = lo + gwarp(); i < hi; i += nwarps()) {
    const int32_t v = b.qv[i];
    const Lanes<W> F = qm[i];
    if (ln == 0) {
      other[v] = F;
      visit[v] = lz<W>();
    }
    if (L == 0) continue;
    const int64_t e0 = g.rowptr[v], e1 = g.rowptr[v + 1];
    if (e1 - e0 > hd.hub_degree) continue;  // k_ms_hub_delta
    const unsigned mine = my_bits(F);
    if (SK == kSigmaU64) {
      df32 acc[2 * W];
      zero_accs(acc);
      psi_range_df<W>(g.colidx, e0, e1, F, succ, b.psi, hd.dense_edges, acc);
      if (b.lane_w) {
        const double contrib =
            warp_sum_f64(finish_df_w<W>(b.psi, b.sigma, v, mine, acc, weights_of<W>(b, v)));
        if (ln == 0) bc[v] += contrib;
      } else {
        df32 contrib = finish_df<W>(b.psi, b.sigma, v, mine, acc);
        contrib = warp_sum_df(contrib);
        if (ln == 0) bc[v] += df_to_double(contrib);
      }
    } else if (SK == kSigmaU64F64) {
      xf64 acc[2 * W];
      psi_range_x<W>(g.colidx, e0, e1, F, succ, b.psi, hd.dense_edges, acc);
      const xf64 contrib = warp_sum_x(
          finish_x<W>(b.psi, b.sigma, v, mine, acc, b.lane_w ? weights_of<W>(b, v) : nullptr));
      if (ln == 0) bc_add_x(bc, v, contrib);
    } else {
      double acc[2 * W];
      zero_accs(acc);
      psi_range_f64<W>(g.colidx, e0, e1, F, succ, b.psi, hd.dense_edges, acc);
      double contrib = b.lane_w ? finish_f64_w<SK, W>(b.psi, b.sigma, v, mine, acc, weights_of<W>(b, v))
                                : finish_f64<SK, W>(b.psi, b.sigma, v, mine, acc);
      contrib = warp_sum_f64(contrib);
      if (ln == 0) bc[v] += contrib;
    }
  }
}

// Hub dependencies at level L over out-edge items; partial psi sums are
// combined in FP64 atomics, the hub's last item finalises delta / psi / bc.
template <int SK, int W>
__global__ void __launch_bounds__(256, W == 1 ? 5 : (W == 2 ? 4 : 3)) k_ms_hub_delta(DevGraph g, MsBuffers b,
                                                                     HubData hd, double* bc) {
  BatchCtl* c = b.ctl;
  const int L = c->level;
  if (L == 0) return;
  const Lanes<W>* __restrict__ succ = mbw<W>(b, L + 1);
  const Lanes<W>* __restrict__ cur = mbw<W>(b, L);
  const int ln = lane_id();
  for (long long it = gwarp(); it < hd.n_out; it += nwarps()) {
    const HubItem I = hd.out_items[it];
    const int32_t h = I.v;
    const Lanes<W> F = cur[h];
    if (!lany(F)) continue;
    unsigned long long* acc = hd.acc + static_cast<int64_t>(I.slot) * (64 * W);
    double part[2 * W];
    if (SK == kSigmaU64) {
      df32 a[2 * W];
      zero_accs(a);
      psi_range_df<W>(g.colidx, I.lo, I.hi, F, succ, b.psi, hd.dense_edges, a);
#pragma unroll
      for (int k = 0; k < 2 * W; ++k) part[k] = df_to_double(a[k]);
    } else if (SK == kSigmaU64F64) {
      xf64 a[2 * W];
      psi_range_x<W>(g.colidx, I.lo, I.hi, F, succ, b.psi, hd.dense_edges, a);
#pragma unroll
      for (int k = 0; k < 2 * W; ++k) part[k] = __longlong_as_double(static_cast<long long>(xf_to_bits(a[k])));
    } else {
      zero_accs(part);
      psi_range_f64<W>(g.colidx, I.lo, I.hi, F, succ, b.psi, hd.dense_edges, part);
    }
#pragma unroll
    for (int k = 0; k < 2 * W; ++k)
      if (part[k] != 0.0) hub_add(acc + 32 * k + ln, part[k]);
    if (!hub_last(hd.cnt + I.slot, I.nitems)) continue;
    double s[2 * W];
#pragma unroll
    for (int k = 0; k < 2 * W; ++k) s[k] = from_bits<double>(atomicExch(acc + 32 * k + ln, 0ull));
    if (ln == 0) hd.cnt[I.slot] = 0u;
    const unsigned mine = my_bits(F);
    if (SK == kSigmaU64) {
      df32 d[2 * W];
#pragma unroll
      for (int k = 0; k < 2 * W; ++k) d[k] = df_from_double(s[k]);
      if (b.lane_w) {
        const double contrib =
            warp_sum_f64(finish_df_w<W>(b.psi, b.sigma, h, mine, d, weights_of<W>(b, h)));
        if (ln == 0) bc[h] += contrib;
      } else {
        df32 contrib = finish_df<W>(b.psi, b.sigma, h, mine, d);
        contrib = warp_sum_df(contrib);
        if (ln == 0) bc[h] += df_to_double(contrib);
      }
    } else if (SK == kSigmaU64F64) {
      xf64 d[2 * W];
#pragma unroll
      for (int k = 0; k < 2 * W; ++k) d[k] = xf_from_bits(static_cast<unsigned long long>(__double_as_longlong(s[k])));
      const xf64 contrib = warp_sum_x(
          finish_x<W>(b.psi, b.sigma, h, mine, d, b.lane_w ? weights_of<W>(b, h) : nullptr));
      if (ln == 0) bc_add_x(bc, h, contrib);
    } else {
      double contrib = b.lane_w ? finish_f64_w<SK, W>(b.psi, b.sigma, h, mine, s, weights_of<W>(b, h))
                                : finish_f64<SK, W>(b.psi, b.sigma, h, mine, s);
      contrib = warp_sum_f64(contrib);
      if (ln == 0) bc[h] += contrib;
    }
  }
}

// ---------------------------------------------------------------------------
// Low-degree variants (segmented warps): a warp takes 32 vertices / list
// entries and streams their concatenated edge lists (seg_gather), instead of
// giving each vertex a whole warp pass.  Same results as k_ms_td_settle,
// k_ms_bu and k_ms_delta.
// ---------------------------------------------------------------------------
template <int SK, int W>
__global__ void __launch_bounds__(256, W == 1 ? 3 : 2) k_ms_td_settle_seg(DevGraph g, MsBuffers b, HubData hd,
                                                          Lanes<W> act) {
  using T = typename Sig<SK>::T;
  BatchCtl* c = b.ctl;
  const unsigned long long lo = c->hi, hi = c->tail;
  const int L = c->level;
  const Lanes<W>* __restrict__ front = mbw<W>(b, L);
  const Lanes<W>* __restrict__ next = mbw<W>(b, L + 1);
  Lanes<W>* qm = lanes_of<W>(b.qm);
  Lanes<W>* visit = lanes_of<W>(b.visit);
  const int ln = lane_id();
  unsigned long long mf = 0, mu = 0, smax = 0;
  for (unsigned long long base = lo + static_cast<unsigned long long>(gwarp()) * kWarp; base < hi;
       base += static_cast<unsigned long long>(nwarps()) * kWarp) {
    const unsigned long long i = base + ln;
    const bool ve = i < hi;
    int32_t w = 0;
    Lanes<W> mask = lz<W>();
    int64_t e0 = 0, deg = 0;
    if (ve) {
      w = b.qv[i];
      mask = next[w];
      e0 = g.in_rowptr[w];
      deg = g.in_rowptr[w + 1] - e0;
      const Lanes<W> nv = lor(visit[w], mask);
      qm[i] = mask;
      visit[w] = nv;
      if (W > 1) b.claim[w] = 0u;
      mf += static_cast<unsigned long long>(g.rowptr[w + 1] - g.rowptr[w]);
      if (leq(nv, act)) mu += static_cast<unsigned long long>(deg);
    }
    const bool mine = ve && deg <= hd.hub_degree;  // hubs: k_ms_hub_pull
    seg_gather<T, T, false, W>(mine, e0, static_cast<int>(mine ? deg : 0), mask, g.in_colidx, front,
                               reinterpret_cast<const T*>(b.sigma),
                               [&](int j, const Lanes<W>& nm, const T (&a)[2 * W]) {
                                 store_sigma<SK, W>(b.sigma, __shfl_sync(kFull, w, j), nm, a, smax);
                               });
  }
  if (SK == kSigmaU64) {
    smax = warp_max_u64(smax);
    if (ln == 0 && smax) atomicMax(&c->sigma_max, smax);
  }
  mf = warp_sum_u64(mf);
  mu = warp_sum_u64(mu);
  if (ln == 0) {
    if (mf) atomicAdd(&c->mf, mf);
    if (mu) atomicAdd(&c->mu_done, mu);
  }
}

template <int SK, int W, bool LF>
__global__ void __launch_bounds__(256, W == 1 ? 3 : 2) k_ms_bu_seg(DevGraph g, MsBuffers b, HubData hd, Lanes<W> act) {
  using T = typename Sig<SK>::T;
  BatchCtl* c = b.ctl;
  const Lanes<W> fl = LF ? frontier_lanes<W>(c) : act;
  const int L = c->level;
  const Lanes<W>* __restrict__ front = mbw<W>(b, L);
  Lanes<W>* next = mbw<W>(b, L + 1);
  Lanes<W>* qm = lanes_of<W>(b.qm);
  Lanes<W>* visit = lanes_of<W>(b.visit);
  const int64_t n = g.n;
  const int ln = lane_id();
  unsigned long long mf = 0, mu = 0, smax = 0;
  for (int64_t base = gwarp() * kWarp; base < n; base += nwarps() * kWarp) {
    const int64_t wme = base + ln;
    Lanes<W> vis = lz<W>();
    int64_t e0 = 0, deg = 0;
    bool cand = false;
    if (wme < n) {
      vis = visit[wme];
      e0 = g.in_rowptr[wme];
      deg = g.in_rowptr[wme + 1] - e0;
      cand = lany(land(lminus(act, vis), fl)) && deg > 0 && deg <= hd.hub_degree;
    }
    Lanes<W> my_nm = lz<W>();
    seg_gather<T, T, false, W>(cand, e0, static_cast<int>(cand ? deg : 0), land(lminus(act, vis), fl),
                               g.in_colidx, front, reinterpret_cast<const T*>(b.sigma),
                               [&](int j, const Lanes<W>& nm, const T (&a)[2 * W]) {
                                 if (lany(nm))
                                   store_sigma<SK, W>(b.sigma, static_cast<int32_t>(base + j), nm,
                                                      a, smax);
                                 if (ln == j) my_nm = nm;
                               });
    const bool app = lany(my_nm);
    const unsigned long long slot = warp_append(app, &c->tail);
    if (app) {
      b.qv[slot] = static_cast<int32_t>(wme);
      qm[slot] = my_nm;
      next[wme] = my_nm;
      const Lanes<W> nv = lor(vis, my_nm);
      visit[wme] = nv;
      mf += static_cast<unsigned long long>(g.rowptr[wme + 1] - g.rowptr[wme]);
      if (leq(nv, act)) mu += static_cast<unsigned long long>(deg);
    }
  }
  if (SK == kSigmaU64) {
    smax = warp_max_u64(smax);
    if (ln == 0 && smax) atomicMax(&c->sigma_max, smax);
  }
  mf = warp_sum_u64(mf);
  mu = warp_sum_u64(mu);
  if (ln == 0) {
    if (mf) atomicAdd(&c->mf, mf);
    if (mu) atomicAdd(&c->mu_done, mu);
  }
}

template <int SK, int W>
__global__ void __launch_bounds__(256, W == 1 ? 3 : 2) k_ms_delta_seg(DevGraph g, MsBuffers b, HubData hd, double* bc) {
  BatchCtl* c = b.ctl;
  const int L = c->level;
  const unsigned long long lo = b.lvl_off[L], hi = b.lvl_off[L + 1];
  const Lanes<W>* __restrict__ succ = mbw<W>(b, L + 1);
  Lanes<W>* other = mbw<W>(b, L);
  const Lanes<W>* qm = lanes_of<W>(b.qm);
  Lanes<W>* visit = lanes_of<W>(b.visit);
  const int ln = lane_id();
  for (unsigned long long base = lo + static_cast<unsigned long long>(gwarp()) * kWarp; base < hi;
       base += static_cast<unsigned long long>(nwarps()) * kWarp) {
    const unsigned long long i = base + ln;
    const bool ve = i < hi;
    int32_t v = 0;
    Lanes<W> F = lz<W>();
    int64_t e0 = 0, deg = 0;
    if (ve) {
      v = b.qv[i];
      F = qm[i];
      other[v] = F;
      visit[v] = lz<W>();
      e0 = g.rowptr[v];
      deg = g.rowptr[v + 1] - e0;
    }
    if (L == 0) continue;
    const bool mine = ve && deg <= hd.hub_degree;  // hubs: k_ms_hub_delta
    const int dg = static_cast<int>(mine ? deg : 0);
    if (SK == kSigmaU64) {
      seg_gather<float2, df32, true, W>(mine, e0, dg, F, g.colidx, succ,
                                        reinterpret_cast<const float2*>(b.psi),
                                        [&](int j, const Lanes<W>&, const df32 (&a)[2 * W]) {
                                          const int32_t vj = __shfl_sync(kFull, v, j);
                                          df32 d[2 * W];
#pragma unroll
                                          for (int k = 0; k < 2 * W; ++k) d[k] = acc_done(a[k]);
                                          df32 contrib = finish_df<W>(b.psi, b.sigma, vj,
                                                                      my_bits(lshfl(F, j)), d);
                                          contrib = warp_sum_df(contrib);
                                          if (ln == 0 && contrib.hi != 0.f) bc[vj] += df_to_double(contrib);
                                        });
    } else if (SK == kSigmaU64F64) {
      seg_gather<unsigned long long, XgAcc<1>, true, W>(
          mine, e0, dg, F, g.colidx, succ, reinterpret_cast<const unsigned long long*>(b.psi),
          [&](int j, const Lanes<W>&, const XgAcc<1> (&a)[2 * W]) {
            const int32_t vj = __shfl_sync(kFull, v, j);
            xf64 d[2 * W];
#pragma unroll
            for (int k = 0; k < 2 * W; ++k) {
              XgAcc<1> t = a[k];  // flushed mid-chunk: renormalise first
              if (k >= Fp64Slots<XgAcc<1>, W>::value) xg_norm(t);
              d[k] = gather_value<W>(t, k);
            }
            const xf64 contrib =
                warp_sum_x(finish_x<W>(b.psi, b.sigma, vj, my_bits(lshfl(F, j)), d, nullptr));
            if (ln == 0) bc_add_x(bc, vj, contrib);
          });
    } else {
      seg_gather<double, double, true, W>(mine, e0, dg, F, g.colidx, succ,
                                          reinterpret_cast<const double*>(b.psi),
                                          [&](int j, const Lanes<W>&, const double (&a)[2 * W]) {
                                            const int32_t vj = __shfl_sync(kFull, v, j);
                                            double contrib = finish_f64<SK, W>(b.psi, b.sigma, vj,
                                                                           my_bits(lshfl(F, j)), a);
                                            contrib = warp_sum_f64(contrib);
                                            if (ln == 0 && contrib != 0.0) bc[vj] += contrib;
                                          });
    }
  }
}

// ---------------------------------------------------------------------------
// Stress centrality (src/centrality/stress.jl:51-77).  For source s the
// reference walks the vertices by decreasing distance and, per w,
//   delta[v] += delta[w] + 1 for every predecessor v of w;
//   delta[w] *= length(P[w]);  stress[w] += delta[w] (w != s),
// all in wrapping Int64.  With D[w] = delta[w] before its multiplication,
//   D[v] = sum over successors c of v of (D[c] + 1),
//   stress[w] += D[w] * |P[w]|,
// where the successors of v are its out-neighbours one level deeper and P[w]
// its in-neighbours one level closer.  The sweep keeps E = D + 1 per (vertex,
// lane) in the path-count rows and uses wrapping uint64 arithmetic, which is
// bit-identical to Julia's Int64.  Level L's step computes E for level L
// (k_st_delta, pull over out-edges against F_{L+1}) and then, with F_L
// complete, the predecessor counts and stress of level L + 1 (k_st_count,
// pull over in-edges against F_L).
// ---------------------------------------------------------------------------

// Per-lane count, over in-edges [e0, e1), of the neighbours u whose mask
// front[u] & want carries the lane (lanes t and t + 32 of this thread).
__device__ __forceinline__ void count_range(const int32_t* __restrict__ ci, int64_t e0, int64_t e1,
                                            uint64_t want, const uint64_t* __restrict__ front,
                                            unsigned long long& c0, unsigned long long& c1) {
  const int ln = lane_id();
  for (int64_t e = e0; e < e1; e += kWarp) {
    const int64_t idx = e + ln;
    uint64_t f = 0;
    if (idx < e1) f = front[ci[idx]] & want;
    if (!__any_sync(kFull, f != 0)) continue;
    c0 += __popc(warp_transpose32(static_cast<uint32_t>(f)));
    c1 += __popc(warp_transpose32(static_cast<uint32_t>(f >> 32)));
  }
}

// stress[w] += sum over the lanes `mine` of w of (E - 1) * count.
__device__ __forceinline__ void stress_finish(const unsigned long long* __restrict__ erow,
                                              uint64_t mask, unsigned long long c0,
                                              unsigned long long c1, unsigned long long* stress,
                                              int32_t w) {
  const int ln = lane_id();
  const unsigned mine = my_bits(mask);
  unsigned long long x = 0;
  if (mine & 1u) x += (erow[ln] - 1ull) * c0;
  if (mine & 2u) x += (erow[32 + ln] - 1ull) * c1;
  x = warp_sum_u64(x);
  if (ln == 0) stress[w] += x;
}

// Level L entries: record F_L, clear visit, and for L >= 1 set E = 1 + sum
// of the successors' E (hubs: k_st_hub_delta).
__global__ void __launch_bounds__(256) k_st_delta(DevGraph g, MsBuffers b, HubData hd) {
  BatchCtl* c = b.ctl;
  const int L = c->level;
  const unsigned long long lo = b.lvl_off[L], hi = b.lvl_off[L + 1];
  const uint64_t* __restrict__ succ = mb_at(b, L + 1);
  uint64_t* other = mb_at(b, L);
  unsigned long long* E = reinterpret_cast<unsigned long long*>(b.sigma);
  const int ln = lane_id();
  for (unsigned long long i = lo + gwarp(); i < hi; i += nwarps()) {
    const int32_t v = b.qv[i];
    const uint64_t F = b.qm[i];
    if (ln == 0) {
      other[v] = F;
      b.visit[v] = 0;
    }
    if (L == 0) continue;
    const int64_t e0 = g.rowptr[v], e1 = g.rowptr[v + 1];
    if (e1 - e0 > hd.hub_degree) continue;
    unsigned long long a[2] = {0ull, 0ull};
    for (int64_t e = e0; e < e1; e += kWarp) {
      const int64_t idx = e + ln;
      int32_t w = 0;
      uint64_t gm = 0;
      if (idx < e1) {
        w = g.colidx[idx];
        gm = succ[w] & F;
      }
      gather_chunk<unsigned long long, unsigned long long, 1>(w, Lanes<1>{{gm}}, E, hd.dense_edges, a);
    }
    const unsigned mine = my_bits(F);
    unsigned long long* row = E + static_cast<int64_t>(v) * 64;
    if (mine & 1u) row[ln] = a[0] + 1ull;
    if (mine & 2u) row[32 + ln] = a[1] + 1ull;
  }
}

__global__ void __launch_bounds__(256) k_st_hub_delta(DevGraph g, MsBuffers b, HubData hd) {
  BatchCtl* c = b.ctl;
  const int L = c->level;
  if (L == 0) return;
  const uint64_t* __restrict__ succ = mb_at(b, L + 1);
  const uint64_t* __restrict__ cur = mb_at(b, L);
  unsigned long long* E = reinterpret_cast<unsigned long long*>(b.sigma);
  const int ln = lane_id();
  for (long long it = gwarp(); it < hd.n_out; it += nwarps()) {
    const HubItem I = hd.out_items[it];
    const int32_t h = I.v;
    const uint64_t F = cur[h];
    if (!F) continue;
    unsigned long long* acc = hd.acc + static_cast<int64_t>(I.slot) * 64;
    unsigned long long a[2] = {0ull, 0ull};
    for (int64_t e = I.lo; e < I.hi; e += kWarp) {
      const int64_t idx = e + ln;
      int32_t w = 0;
      uint64_t gm = 0;
      if (idx < I.hi) {
        w = g.colidx[idx];
        gm = succ[w] & F;
      }
      gather_chunk<unsigned long long, unsigned long long, 1>(w, Lanes<1>{{gm}}, E, hd.dense_edges, a);
    }
    if (a[0]) atomicAdd(acc + ln, a[0]);
    if (a[1]) atomicAdd(acc + 32 + ln, a[1]);
    if (!hub_last(hd.cnt + I.slot, I.nitems)) continue;
    const unsigned long long s0 = atomicExch(acc + ln, 0ull);
    const unsigned long long s1 = atomicExch(acc + 32 + ln, 0ull);
    if (ln == 0) hd.cnt[I.slot] = 0u;
    const unsigned mine = my_bits(F);
    unsigned long long* row = E + static_cast<int64_t>(h) * 64;
    if (mine & 1u) row[ln] = s0 + 1ull;
    if (mine & 2u) row[32 + ln] = s1 + 1ull;
  }
}

// Level L + 1 entries (after k_st_delta of level L wrote F_L): predecessor
// counts over in-edges and the stress contribution (hubs: k_st_hub_count).
__global__ void __launch_bounds__(256) k_st_count(DevGraph g, MsBuffers b, HubData hd,
                                                  unsigned long long* stress) {
  BatchCtl* c = b.ctl;
  const int L = c->level;
  if (L + 1 > c->maxlevel) return;
  const unsigned long long lo = b.lvl_off[L + 1], hi = b.lvl_off[L + 2];
  const uint64_t* __restrict__ front = mb_at(b, L);
  const unsigned long long* E = reinterpret_cast<const unsigned long long*>(b.sigma);
  for (unsigned long long i = lo + gwarp(); i < hi; i += nwarps()) {
    const int32_t w = b.qv[i];
    const uint64_t F = b.qm[i];
    const int64_t e0 = g.in_rowptr[w], e1 = g.in_rowptr[w + 1];
    if (e1 - e0 > hd.hub_degree) continue;
    unsigned long long c0 = 0, c1 = 0;
    count_range(g.in_colidx, e0, e1, F, front, c0, c1);
    stress_finish(E + static_cast<int64_t>(w) * 64, F, c0, c1, stress, w);
  }
}

__global__ void __launch_bounds__(256) k_st_hub_count(DevGraph g, MsBuffers b, HubData hd,
                                                      unsigned long long* stress) {
  BatchCtl* c = b.ctl;
  const int L = c->level;
  if (L + 1 > c->maxlevel) return;
  const uint64_t* __restrict__ front = mb_at(b, L);
  const uint64_t* __restrict__ nxt = mb_at(b, L + 1);
  const unsigned long long* E = reinterpret_cast<const unsigned long long*>(b.sigma);
  const int ln = lane_id();
  for (long long it = gwarp(); it < hd.n_in; it += nwarps()) {
    const HubItem I = hd.in_items[it];
    const int32_t h = I.v;
    const uint64_t F = nxt[h];
    if (!F) continue;
    unsigned long long* acc = hd.acc + static_cast<int64_t>(I.slot) * 64;
    unsigned long long c0 = 0, c1 = 0;
    count_range(g.in_colidx, I.lo, I.hi, F, front, c0, c1);
    if (c0) atomicAdd(acc + ln, c0);
    if (c1) atomicAdd(acc + 32 + ln, c1);
    if (!hub_last(hd.cnt + I.slot, I.nitems)) continue;
    const unsigned long long s0 = atomicExch(acc + ln, 0ull);
    const unsigned long long s1 = atomicExch(acc + 32 + ln, 0ull);
    if (ln == 0) hd.cnt[I.slot] = 0u;
    stress_finish(E + static_cast<int64_t>(h) * 64, F, s0, s1, stress, h);
  }
}

__global__ void k_ms_back_advance(MsBuffers b) { b.ctl->level -= 1; }

// End of a Brandes batch: the backward sweep cleared visit for every listed
// vertex; clear the dense masks of levels 0 and 1 that remain.
template <int W>
__global__ void k_ms_cleanup(MsBuffers b) {
  const unsigned long long lo = b.lvl_off[0], hi = b.lvl_off[2];
  Lanes<W>* m0 = lanes_of<W>(b.mb[0]);
  Lanes<W>* m1 = lanes_of<W>(b.mb[1]);
  Lanes<W>* visit = lanes_of<W>(b.visit);
  for (unsigned long long i = lo + blockIdx.x * blockDim.x + threadIdx.x; i < hi;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
    const int32_t v = b.qv[i];
    m0[v] = lz<W>();
    m1[v] = lz<W>();
    visit[v] = lz<W>();
  }
}

// End of a distance-only batch: clear every listed vertex.
__global__ void k_ms_cleanup_all(MsBuffers b) {
  const unsigned long long hi = b.ctl->tail;
  for (unsigned long long i = blockIdx.x * blockDim.x + threadIdx.x; i < hi;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
    const int32_t v = b.qv[i];
    b.mb[0][v] = 0;
    b.mb[1][v] = 0;
    b.visit[v] = 0;
  }
}

// Export of a one-word forward sweep with path counts (before the batch is
// cleaned up): every listed (v, lanes) at level L gives, for each of its
// lanes l, sigma_out[l * ld + v] = the path count as binary64 (exact below
// 2^53; the uint64 count rounded to nearest above) and dist_out[l * ld + v] =
// L.  Thread t of the warp that owns an entry writes lanes t and t + 32.
// These are DijkstraState.pathcounts and .dists of
// dijkstra_shortest_paths(g, s) with unit weights
// (src/shortestpaths/dijkstra.jl:59-141); vertices a lane never lists keep
// the caller's prefill (0 and LGBC_UNREACHED).
template <int SK>
__global__ void k_ms_export(MsBuffers b, double* sigma_out, int32_t* dist_out, int64_t ld) {
  using T = typename Sig<SK>::T;
  const BatchCtl* c = b.ctl;
  const int maxl = c->maxlevel;
  const unsigned long long total = b.lvl_off[maxl + 1];
  const T* sigma = reinterpret_cast<const T*>(b.sigma);
  const int ln = lane_id();
  for (unsigned long long i = gwarp(); i < total; i += nwarps()) {
    // the level of entry i: the largest L with lvl_off[L] <= i
    int lo = 0, hi = maxl;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (b.lvl_off[mid] <= i) lo = mid;
      else hi = mid - 1;
    }
    const int32_t v = b.qv[i];
    const uint64_t F = b.qm[i];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int l = 32 * k + ln;
      if ((F >> l) & 1ull) {
        const int64_t o = static_cast<int64_t>(l) * ld + v;
        sigma_out[o] = sigma_f64(sigma[static_cast<int64_t>(v) * 64 + l]);
        if (dist_out) dist_out[o] = lo;
      }
    }
  }
}

// Distance statistics of every lane after a forward sweep: cnt[lane] +=
// vertices the lane reached at levels >= 1, dsum[lane] += the sum of those
// levels, dmax[lane] = max(dmax[lane], deepest level).  A warp loads 32 list
// entries, then walks them by broadcast; thread t owns lanes t and t + 32;
// block sums go out with one atomic per lane per block.
//
// The dependency mass of a source follows from them exactly:
//   sum_{v != s} delta_s(v) = sum_{t reachable from s, t != s} (d(s, t) - 1)
// (delta_s(v) = sum_t sigma_st(v) / sigma_st, and sum_v sigma_st(v) / sigma_st
// is the number of interior vertices of a shortest s-t path).
__global__ void __launch_bounds__(256) k_ms_level_stats(MsBuffers b, unsigned long long* cnt,
                                                        unsigned long long* dsum, int* dmax) {
  __shared__ unsigned long long pc[64], ps[64];
  __shared__ int pm[64];
  const int ln = lane_id();
  if (threadIdx.x < 64) {
    pc[threadIdx.x] = 0ull;
    ps[threadIdx.x] = 0ull;
    pm[threadIdx.x] = 0;
  }
  __syncthreads();
  const int maxl = b.ctl->maxlevel;
  const unsigned long long lo = b.lvl_off[1], hi = b.lvl_off[maxl + 1];
  unsigned long long c0 = 0, c1 = 0, s0 = 0, s1 = 0;
  int m0 = 0, m1 = 0;
  const unsigned long long stride = static_cast<unsigned long long>(nwarps()) * 32;
  for (unsigned long long base = lo + static_cast<unsigned long long>(gwarp()) * 32; base < hi;
       base += stride) {
    const unsigned long long i = base + ln;
    uint64_t m = 0;
    int lev = 0;
    if (i < hi) {
      m = b.qm[i];
      int l = 1, r = maxl;  // largest L in [1, maxl] with lvl_off[L] <= i
      while (l < r) {
        const int mid = (l + r + 1) >> 1;
        if (b.lvl_off[mid] <= i) l = mid; else r = mid - 1;
      }
      lev = l;
    }
    for (int j = 0; j < 32; ++j) {
      const uint64_t mj = shfl_u64(m, j);
      const int lj = __shfl_sync(kFull, lev, j);
      if ((mj >> ln) & 1ull) {
        c0 += 1;
        s0 += static_cast<unsigned long long>(lj);
        m0 = max(m0, lj);
      }
      if ((mj >> (32 + ln)) & 1ull) {
        c1 += 1;
        s1 += static_cast<unsigned long long>(lj);
        m1 = max(m1, lj);
      }
    }
  }
  if (c0) {
    atomicAdd(&pc[ln], c0);
    atomicAdd(&ps[ln], s0);
    atomicMax(&pm[ln], m0);
  }
  if (c1) {
    atomicAdd(&pc[32 + ln], c1);
    atomicAdd(&ps[32 + ln], s1);
    atomicMax(&pm[32 + ln], m1);
  }
  __syncthreads();
  if (threadIdx.x < 64 && pc[threadIdx.x]) {
    atomicAdd(cnt + threadIdx.x, pc[threadIdx.x]);
    atomicAdd(dsum + threadIdx.x, ps[threadIdx.x]);
    atomicMax(dmax + threadIdx.x, pm[threadIdx.x]);
  }
}

// Batch initialisation with explicit seeds: seed i puts vertex seed_v[i] at
// level 0 of the lanes in its lane set (W words at seed_mask[i * W]).  Used
// for disjoint unions of graphs, where a lane may hold one source in every
// component: BFS trees of different components never meet, so each component
// sees a single-source traversal.  Seed vertices must be distinct (a vertex
// that starts several lanes is one seed with several bits).  The host zeroes
// the control block first.
template <int SK, int W>
__global__ void k_ms_init_seeds(DevGraph g, MsBuffers b, const int32_t* seed_v,
                                const uint64_t* seed_mask, long long nseeds, int32_t* dist,
                                int64_t ld) {
  using T = typename Sig<SK>::T;
  const Lanes<W>* masks = lanes_of<W>(seed_mask);
  Lanes<W>* front = lanes_of<W>(b.mb[0]);
  Lanes<W>* visit = lanes_of<W>(b.visit);
  Lanes<W>* qm = lanes_of<W>(b.qm);
  unsigned long long mf = 0;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < nseeds;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int32_t v = seed_v[i];
    const Lanes<W> m = masks[i];
    front[v] = m;
    visit[v] = lor(visit[v], m);
    b.qv[i] = v;
    qm[i] = m;
#pragma unroll
    for (int j = 0; j < W; ++j) {
      for (uint64_t r = m.w[j]; r; r &= r - 1) {
        const int l = 64 * j + __ffsll(static_cast<long long>(r)) - 1;
        if (SK != kSigmaNone)
          reinterpret_cast<T*>(b.sigma)[static_cast<int64_t>(v) * (64 * W) + l] = T(1);
        if (dist) dist[static_cast<int64_t>(l) * ld + v] = 0;
      }
    }
    mf += static_cast<unsigned long long>(g.rowptr[v + 1] - g.rowptr[v]);
  }
  mf = warp_sum_u64(mf);
  if (lane_id() == 0 && mf) atomicAdd(&b.ctl->mf_cur, mf);
}

// Union batches: lanes that hold no source in a component can never reach
// its vertices; marking them visited there keeps bottom-up levels from
// rescanning those vertices.  Block k covers component k; seg_mark holds W
// words per component.
template <int W>
__global__ void k_ms_premark(uint64_t* visit_words, const int64_t* seg_off, const uint64_t* seg_mark,
                             int64_t nseg) {
  Lanes<W>* visit = lanes_of<W>(visit_words);
  const Lanes<W>* marks = lanes_of<W>(seg_mark);
  for (int64_t k = blockIdx.x; k < nseg; k += gridDim.x) {
    const Lanes<W> m = marks[k];
    for (int64_t v = seg_off[k] + threadIdx.x; v < seg_off[k + 1]; v += blockDim.x) visit[v] = m;
  }
}

__global__ void k_ms_init_seeds_ctl(MsBuffers b, long long nseeds, unsigned long long cap,
                                    unsigned long long sigma_limit) {
  BatchCtl* c = b.ctl;
  c->lo = 0;
  c->hi = static_cast<unsigned long long>(nseeds);
  c->tail = static_cast<unsigned long long>(nseeds);
  c->mf = 0;
  c->mu_done = 0;
  c->cap = cap;
  c->level = 0;
  c->maxlevel = 0;
  c->done = 0;
  c->overflow_list = 0;
  c->overflow_sigma = 0;
  c->mode = 0;
  c->sigma_max = 1;
  c->sigma_limit = sigma_limit;
  c->td_levels = 0;
  c->bu_levels = 0;
  c->runaway = 0;
  for (int j = 0; j < kMaxWords; ++j) {
    c->front_union[j] = ~0ull;  // every lane may be seeded
    c->next_union[j] = 0ull;
  }
  b.lvl_off[0] = 0;
  b.lvl_off[1] = static_cast<unsigned long long>(nseeds);
}

// A multi-word batch (Brandes batches only: no distance rows).
template <int W>
void init_wide(cudaStream_t s, const DevGraph& g, const MsBuffers& b, int nlanes, const Lanes<W>& a,
               int sigma_kind, unsigned long long sigma_limit) {
  switch (sigma_kind) {
    case kSigmaU64:
      k_ms_init<kSigmaU64, W><<<1, kWideLanes, 0, s>>>(g, b, nlanes, a, b.cap, sigma_limit, nullptr, 0);
      break;
    case kSigmaF64:
      k_ms_init<kSigmaF64, W><<<1, kWideLanes, 0, s>>>(g, b, nlanes, a, b.cap, ~0ull, nullptr, 0);
      break;
    default:
      k_ms_init<kSigmaNone, W><<<1, kWideLanes, 0, s>>>(g, b, nlanes, a, b.cap, ~0ull, nullptr, 0);
      break;
  }
}

}  // namespace

int ms_init(cudaStream_t s, const DevGraph& g, const MsBuffers& b, int nlanes, int sigma_kind,
            unsigned long long sigma_limit, int32_t* dist, int64_t dist_ld) {
  sigma_kind = fwd_kind(sigma_kind);
  const LaneSet act = lane_set(nlanes, b.words);
  if (b.words == 4) {
    init_wide<4>(s, g, b, nlanes, lane_cast<4>(act), sigma_kind, sigma_limit);
    return 1;
  }
  if (b.words == 2) {
    init_wide<2>(s, g, b, nlanes, lane_cast<2>(act), sigma_kind, sigma_limit);
    return 1;
  }
  const Lanes<1> a = lane_cast<1>(act);
  switch (sigma_kind) {
    case kSigmaU64:
      k_ms_init<kSigmaU64, 1><<<1, kWideLanes, 0, s>>>(g, b, nlanes, a, b.cap, sigma_limit, dist, dist_ld);
      break;
    case kSigmaF64:
      k_ms_init<kSigmaF64, 1><<<1, kWideLanes, 0, s>>>(g, b, nlanes, a, b.cap, ~0ull, dist, dist_ld);
      break;
    default:
      k_ms_init<kSigmaNone, 1><<<1, kWideLanes, 0, s>>>(g, b, nlanes, a, b.cap, ~0ull, dist, dist_ld);
      break;
  }
  return 1;
}

namespace {

template <int W>
void init_seeds_w(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const MsBuffers& b,
                  const int32_t* seed_v, const uint64_t* seed_mask, int64_t nseeds, int sigma_kind,
                  unsigned long long sigma_limit, int32_t* dist, int64_t dist_ld) {
  const int grid = static_cast<int>(std::min<int64_t>((nseeds + 255) / 256, c.grid));
  switch (sigma_kind) {
    case kSigmaU64:
      k_ms_init_seeds<kSigmaU64, W><<<grid, 256, 0, s>>>(g, b, seed_v, seed_mask, nseeds, dist, dist_ld);
      k_ms_init_seeds_ctl<<<1, 1, 0, s>>>(b, nseeds, b.cap, sigma_limit);
      break;
    case kSigmaF64:
      k_ms_init_seeds<kSigmaF64, W><<<grid, 256, 0, s>>>(g, b, seed_v, seed_mask, nseeds, dist, dist_ld);
      k_ms_init_seeds_ctl<<<1, 1, 0, s>>>(b, nseeds, b.cap, ~0ull);
      break;
    default:
      k_ms_init_seeds<kSigmaNone, W><<<grid, 256, 0, s>>>(g, b, seed_v, seed_mask, nseeds, dist, dist_ld);
      k_ms_init_seeds_ctl<<<1, 1, 0, s>>>(b, nseeds, b.cap, ~0ull);
      break;
  }
}

}  // namespace

int ms_init_seeds(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const MsBuffers& b,
                  const int32_t* seed_v, const uint64_t* seed_mask, int64_t nseeds, int sigma_kind,
                  unsigned long long sigma_limit, int32_t* dist, int64_t dist_ld) {
  sigma_kind = fwd_kind(sigma_kind);
  cudaMemsetAsync(b.ctl, 0, sizeof(BatchCtl), s);
  if (b.words == 4)
    init_seeds_w<4>(c, s, g, b, seed_v, seed_mask, nseeds, sigma_kind, sigma_limit, nullptr, 0);
  else if (b.words == 2)
    init_seeds_w<2>(c, s, g, b, seed_v, seed_mask, nseeds, sigma_kind, sigma_limit, nullptr, 0);
  else
    init_seeds_w<1>(c, s, g, b, seed_v, seed_mask, nseeds, sigma_kind, sigma_limit, dist, dist_ld);
  return 2;
}

int ms_premark(const LaunchCfg& c, cudaStream_t s, const MsBuffers& b, const int64_t* seg_off,
               const uint64_t* seg_mark, int64_t nseg) {
  if (b.words == 4)
    k_ms_premark<4><<<c.grid, c.block, 0, s>>>(b.visit, seg_off, seg_mark, nseg);
  else if (b.words == 2)
    k_ms_premark<2><<<c.grid, c.block, 0, s>>>(b.visit, seg_off, seg_mark, nseg);
  else
    k_ms_premark<1><<<c.grid, c.block, 0, s>>>(b.visit, seg_off, seg_mark, nseg);
  return 1;
}

namespace {

// The segmented low-degree kernels exist for one- and two-word batches.
template <int W> constexpr bool has_seg() { return W < 4; }

template <int W, bool LF>
int topdown_w(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const MsBuffers& b,
              const HubData& hd, const Lanes<W>& act, int sigma_kind, int32_t* dist,
              int64_t dist_ld) {
  int launches = 0;
  k_ms_td_discover<W><<<c.grid, c.block, 0, s>>>(g, b, hd);
  ++launches;
  if (hd.n_out > 0) {
    k_ms_hub_discover<W><<<c.grid, c.block, 0, s>>>(g, b, hd);
    ++launches;
  }
  if (sigma_kind == kSigmaNone) {
    if constexpr (W == 1) {
      if (dist)
        k_ms_td_settle<kSigmaNone, true, 1><<<c.grid, c.block, 0, s>>>(g, b, hd, act, dist, dist_ld);
      else
        k_ms_td_settle<kSigmaNone, false, 1><<<c.grid, c.block, 0, s>>>(g, b, hd, act, dist, dist_ld);
    } else {
      k_ms_td_settle<kSigmaNone, false, W><<<c.grid, c.block, 0, s>>>(g, b, hd, act, nullptr, 0);
    }
  } else if (sigma_kind == kSigmaU64) {
    if (has_seg<W>() && hd.segmented) {
      if constexpr (has_seg<W>()) k_ms_td_settle_seg<kSigmaU64, W><<<c.grid, c.block, 0, s>>>(g, b, hd, act);
    } else
      k_ms_td_settle<kSigmaU64, false, W><<<c.grid, c.block, 0, s>>>(g, b, hd, act, dist, dist_ld);
    if (hd.n_in > 0) {
      k_ms_hub_pull<kSigmaU64, false, false, W, false><<<c.grid, c.block, 0, s>>>(g, b, hd, act, dist,
                                                                                 dist_ld);
      ++launches;
    }
  } else {
    if (has_seg<W>() && hd.segmented) {
      if constexpr (has_seg<W>()) k_ms_td_settle_seg<kSigmaF64, W><<<c.grid, c.block, 0, s>>>(g, b, hd, act);
    } else
      k_ms_td_settle<kSigmaF64, false, W><<<c.grid, c.block, 0, s>>>(g, b, hd, act, dist, dist_ld);
    if (hd.n_in > 0) {
      k_ms_hub_pull<kSigmaF64, false, false, W, false><<<c.grid, c.block, 0, s>>>(g, b, hd, act, dist,
                                                                                 dist_ld);
      ++launches;
    }
  }
  ++launches;
  k_ms_clear_front<W, LF><<<c.grid, c.block, 0, s>>>(b);
  return launches + 1;
}

template <int W, bool LF>
int bottomup_w(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const MsBuffers& b,
               const HubData& hd, const Lanes<W>& act, int sigma_kind, int32_t* dist,
               int64_t dist_ld) {
  int launches = 1;
  if (sigma_kind == kSigmaNone) {
    if constexpr (W == 1) {
      if (dist)
        k_ms_bu<kSigmaNone, true, 1, LF><<<c.grid, c.block, 0, s>>>(g, b, hd, act, dist, dist_ld);
      else
        k_ms_bu<kSigmaNone, false, 1, LF><<<c.grid, c.block, 0, s>>>(g, b, hd, act, dist, dist_ld);
      if (hd.n_in > 0) {
        if (dist)
          k_ms_hub_pull<kSigmaNone, true, true, 1, LF><<<c.grid, c.block, 0, s>>>(g, b, hd, act, dist,
                                                                                 dist_ld);
        else
          k_ms_hub_pull<kSigmaNone, false, true, 1, LF><<<c.grid, c.block, 0, s>>>(g, b, hd, act, dist,
                                                                                  dist_ld);
        ++launches;
      }
    } else {
      k_ms_bu<kSigmaNone, false, W, LF><<<c.grid, c.block, 0, s>>>(g, b, hd, act, nullptr, 0);
      if (hd.n_in > 0) {
        k_ms_hub_pull<kSigmaNone, false, true, W, LF><<<c.grid, c.block, 0, s>>>(g, b, hd, act, nullptr,
                                                                                0);
        ++launches;
      }
    }
  } else if (sigma_kind == kSigmaU64) {
    if (has_seg<W>() && hd.segmented) {
      if constexpr (has_seg<W>()) k_ms_bu_seg<kSigmaU64, W, LF><<<c.grid, c.block, 0, s>>>(g, b, hd, act);
    } else
      k_ms_bu<kSigmaU64, false, W, LF><<<c.grid, c.block, 0, s>>>(g, b, hd, act, dist, dist_ld);
    if (hd.n_in > 0) {
      k_ms_hub_pull<kSigmaU64, false, true, W, LF><<<c.grid, c.block, 0, s>>>(g, b, hd, act, dist,
                                                                             dist_ld);
      ++launches;
    }
  } else {
    if (has_seg<W>() && hd.segmented) {
      if constexpr (has_seg<W>()) k_ms_bu_seg<kSigmaF64, W, LF><<<c.grid, c.block, 0, s>>>(g, b, hd, act);
    } else
      k_ms_bu<kSigmaF64, false, W, LF><<<c.grid, c.block, 0, s>>>(g, b, hd, act, dist, dist_ld);
    if (hd.n_in > 0) {
      k_ms_hub_pull<kSigmaF64, false, true, W, LF><<<c.grid, c.block, 0, s>>>(g, b, hd, act, dist,
                                                                             dist_ld);
      ++launches;
    }
  }
  k_ms_clear_front<W, LF><<<c.grid, c.block, 0, s>>>(b);
  return launches + 1;
}

template <int W>
int backward_body_w(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const MsBuffers& b,
                    const HubData& hd, int sigma_kind, double* bc) {
  int launches = 2;
  k_ms_back_clear<W><<<c.grid, c.block, 0, s>>>(b);
  // the segmented variant has no weighted finalisation
  const bool seg = has_seg<W>() && hd.segmented && !b.lane_w;
  if (sigma_kind == kSigmaU64F64) {
    if (seg) {
      if constexpr (has_seg<W>()) k_ms_delta_seg<kSigmaU64F64, W><<<c.grid, c.block, 0, s>>>(g, b, hd, bc);
    } else
      k_ms_delta<kSigmaU64F64, W><<<c.grid, c.block, 0, s>>>(g, b, hd, bc);
    if (hd.n_out > 0) {
      k_ms_hub_delta<kSigmaU64F64, W><<<c.grid, c.block, 0, s>>>(g, b, hd, bc);
      ++launches;
    }
  } else if (sigma_kind == kSigmaF64) {
    if (seg) {
      if constexpr (has_seg<W>()) k_ms_delta_seg<kSigmaF64, W><<<c.grid, c.block, 0, s>>>(g, b, hd, bc);
    } else
      k_ms_delta<kSigmaF64, W><<<c.grid, c.block, 0, s>>>(g, b, hd, bc);
    if (hd.n_out > 0) {
      k_ms_hub_delta<kSigmaF64, W><<<c.grid, c.block, 0, s>>>(g, b, hd, bc);
      ++launches;
    }
  } else {
    if (seg) {
      if constexpr (has_seg<W>()) k_ms_delta_seg<kSigmaU64, W><<<c.grid, c.block, 0, s>>>(g, b, hd, bc);
    } else
      k_ms_delta<kSigmaU64, W><<<c.grid, c.block, 0, s>>>(g, b, hd, bc);
    if (hd.n_out > 0) {
      k_ms_hub_delta<kSigmaU64, W><<<c.grid, c.block, 0, s>>>(g, b, hd, bc);
      ++launches;
    }
  }
  return launches;
}

}  // namespace

int ms_topdown(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const MsBuffers& b,
               const HubData& hd, const LaneSet& act, int sigma_kind, int32_t* dist,
               int64_t dist_ld) {
  sigma_kind = fwd_kind(sigma_kind);
  if (b.words == 4)
    return b.lane_filter
               ? topdown_w<4, true>(c, s, g, b, hd, lane_cast<4>(act), sigma_kind, dist, dist_ld)
               : topdown_w<4, false>(c, s, g, b, hd, lane_cast<4>(act), sigma_kind, dist, dist_ld);
  if (b.words == 2)
    return b.lane_filter
               ? topdown_w<2, true>(c, s, g, b, hd, lane_cast<2>(act), sigma_kind, dist, dist_ld)
               : topdown_w<2, false>(c, s, g, b, hd, lane_cast<2>(act), sigma_kind, dist, dist_ld);
  return b.lane_filter
             ? topdown_w<1, true>(c, s, g, b, hd, lane_cast<1>(act), sigma_kind, dist, dist_ld)
             : topdown_w<1, false>(c, s, g, b, hd, lane_cast<1>(act), sigma_kind, dist, dist_ld);
}

int ms_bottomup(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const MsBuffers& b,
                const HubData& hd, const LaneSet& act, int sigma_kind, int32_t* dist,
                int64_t dist_ld) {
  sigma_kind = fwd_kind(sigma_kind);
  if (b.words == 4)
    return b.lane_filter
               ? bottomup_w<4, true>(c, s, g, b, hd, lane_cast<4>(act), sigma_kind, dist, dist_ld)
               : bottomup_w<4, false>(c, s, g, b, hd, lane_cast<4>(act), sigma_kind, dist, dist_ld);
  if (b.words == 2)
    return b.lane_filter
               ? bottomup_w<2, true>(c, s, g, b, hd, lane_cast<2>(act), sigma_kind, dist, dist_ld)
               : bottomup_w<2, false>(c, s, g, b, hd, lane_cast<2>(act), sigma_kind, dist, dist_ld);
  return b.lane_filter
             ? bottomup_w<1, true>(c, s, g, b, hd, lane_cast<1>(act), sigma_kind, dist, dist_ld)
             : bottomup_w<1, false>(c, s, g, b, hd, lane_cast<1>(act), sigma_kind, dist, dist_ld);
}

int ms_advance(cudaStream_t s, const DevGraph& g, const MsBuffers& b) {
  k_ms_advance<<<1, 1, 0, s>>>(b, g.n);
  return 1;
}

int ms_begin_backward(cudaStream_t s, const MsBuffers& b) {
  k_ms_begin_backward<<<1, 1, 0, s>>>(b);
  return 1;
}

int ms_backward_level(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const MsBuffers& b,
                      const HubData& hd, int sigma_kind, double* bc) {
  const int launches = ms_backward_body(c, s, g, b, hd, sigma_kind, bc);
  k_ms_back_advance<<<1, 1, 0, s>>>(b);
  return launches + 1;
}

int ms_backward_body(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const MsBuffers& b,
                     const HubData& hd, int sigma_kind, double* bc) {
  if (b.words == 4) return backward_body_w<4>(c, s, g, b, hd, sigma_kind, bc);
  if (b.words == 2) return backward_body_w<2>(c, s, g, b, hd, sigma_kind, bc);
  return backward_body_w<1>(c, s, g, b, hd, sigma_kind, bc);
}

int loop_arm(cudaStream_t s, const MsBuffers& b, const LoopParams& lp) {
  k_loop_arm<<<1, 1, 0, s>>>(b, lp);
  return 1;
}

int loop_advance(cudaStream_t s, const MsBuffers& b, const LoopParams& lp) {
  k_loop_advance<<<1, 1, 0, s>>>(b, lp);
  return 1;
}

int loop_back_arm(cudaStream_t s, const MsBuffers& b, const LoopParams& lp) {
  k_loop_back_arm<<<1, 1, 0, s>>>(b, lp);
  return 1;
}

int loop_back_advance(cudaStream_t s, const MsBuffers& b, const LoopParams& lp) {
  k_loop_back_advance<<<1, 1, 0, s>>>(b, lp);
  return 1;
}

int st_backward_level(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const MsBuffers& b,
                      const HubData& hd, unsigned long long* stress) {
  int launches = 4;
  k_ms_back_clear<1><<<c.grid, c.block, 0, s>>>(b);
  k_st_delta<<<c.grid, c.block, 0, s>>>(g, b, hd);
  if (hd.n_out > 0) {
    k_st_hub_delta<<<c.grid, c.block, 0, s>>>(g, b, hd);
    ++launches;
  }
  k_st_count<<<c.grid, c.block, 0, s>>>(g, b, hd, stress);
  if (hd.n_in > 0) {
    k_st_hub_count<<<c.grid, c.block, 0, s>>>(g, b, hd, stress);
    ++launches;
  }
  k_ms_back_advance<<<1, 1, 0, s>>>(b);
  return launches;
}

int ms_cleanup(const LaunchCfg& c, cudaStream_t s, const MsBuffers& b) {
  if (b.words == 4)
    k_ms_cleanup<4><<<c.grid, c.block, 0, s>>>(b);
  else if (b.words == 2)
    k_ms_cleanup<2><<<c.grid, c.block, 0, s>>>(b);
  else
    k_ms_cleanup<1><<<c.grid, c.block, 0, s>>>(b);
  return 1;
}

int ms_level_stats(const LaunchCfg& c, cudaStream_t s, const MsBuffers& b, const LevelStats& st) {
  k_ms_level_stats<<<c.sms * 2, 256, 0, s>>>(b, st.cnt, st.dsum, st.dmax);
  return 1;
}

int ms_cleanup_all(const LaunchCfg& c, cudaStream_t s, const MsBuffers& b) {
  k_ms_cleanup_all<<<c.grid, c.block, 0, s>>>(b);
  return 1;
}

int ms_export(const LaunchCfg& c, cudaStream_t s, const MsBuffers& b, int sigma_kind,
              double* sigma_out, int32_t* dist_out, int64_t ld) {
  if (sigma_kind == kSigmaF64)
    k_ms_export<kSigmaF64><<<c.grid, c.block, 0, s>>>(b, sigma_out, dist_out, ld);
  else
    k_ms_export<kSigmaU64><<<c.grid, c.block, 0, s>>>(b, sigma_out, dist_out, ld);
  return 1;
}

int ms_reset_all(cudaStream_t s, const DevGraph& g, const MsBuffers& b) {
  const size_t bytes = static_cast<size_t>(g.n) * sizeof(uint64_t) * kMaxWords;
  cudaMemsetAsync(b.visit, 0, bytes, s);
  cudaMemsetAsync(b.mb[0], 0, bytes, s);
  cudaMemsetAsync(b.mb[1], 0, bytes, s);
  if (b.claim) cudaMemsetAsync(b.claim, 0, static_cast<size_t>(g.n) * sizeof(unsigned), s);
  return 0;
}

}  // namespace lgbc
