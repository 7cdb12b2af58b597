// ingest.cu -- graph ingest on the device: a CSR built from an edge list.
//
// Replaces the host-side flattening of add_edge!-built adjacency lists for
// large graphs: SimpleGraph / SimpleDiGraph keep every neighbour list sorted
// and free of duplicates (src/SimpleGraphs/simplegraph.jl:445-461,
// simpledigraph.jl:414-429), and an undirected self-loop is stored once.
// Every arc becomes a 64-bit key (u << B) | v with B = bit width of n; the keys
// are sorted by an LSD radix sort (8-bit digits, stable tile scatter), equal
// keys collapse, and the row starts come from a histogram of u and a scan.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lgbc_kernels.h"

namespace lgbc {
namespace {

constexpr int kRsThreads = 256;
constexpr int kRsItems = 16;                       // keys per thread per tile
constexpr int kRsTile = kRsThreads * kRsItems;     // 4096
constexpr int kRsWarps = kRsThreads / 32;
constexpr unsigned long long kSentinel = ~0ull;    // "no arc" (sorts last)

// ---- arcs --------------------------------------------------------------------
// Undirected: slot 2i = (u, v), slot 2i + 1 = (v, u), or the sentinel for a
// self-loop (stored once).  Directed: slot i = (u, v).  *bad |= 1 when an id
// is outside [0, n).
__global__ void k_make_keys(const int32_t* src, const int32_t* dst, int64_t m, int64_t n, int B,
                            int directed, unsigned long long* keys, int* bad) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < m;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int32_t u = src[i], v = dst[i];
    const bool ok = u >= 0 && u < n && v >= 0 && v < n;
    if (!ok) atomicOr(bad, 1);
    const unsigned long long uu = ok ? static_cast<unsigned long long>(u) : 0ull;
    const unsigned long long vv = ok ? static_cast<unsigned long long>(v) : 0ull;
    if (directed) {
      keys[i] = ok ? ((uu << B) | vv) : kSentinel;
    } else {
      keys[2 * i] = ok ? ((uu << B) | vv) : kSentinel;
      keys[2 * i + 1] = (ok && u != v) ? ((vv << B) | uu) : kSentinel;
    }
  }
}

// Swap the two halves of every key: (u, v) -> (v, u) (the in-CSR of a digraph).
__global__ void k_swap_keys(const unsigned long long* in, int64_t count, int B,
                            unsigned long long* out) {
  const unsigned long long mask = (1ull << B) - 1ull;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const unsigned long long k = in[i];
    out[i] = ((k & mask) << B) | (k >> B);
  }
}

// ---- LSD radix sort, one 8-bit digit per pass ------------------------------
// hist[d * tiles + t] = keys of tile t with digit d.
__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const unsigned long long* keys, int64_t count,
                                                        int shift, int64_t tiles, uint32_t* hist) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0u;
  __syncthreads();
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kRsTile;
  for (int r = 0; r < kRsItems; ++r) {
    const int64_t i = base + r * kRsThreads + threadIdx.x;
    if (i < count) atomicAdd(&h[(keys[i] >> shift) & 255ull], 1u);
  }
  __syncthreads();
  hist[static_cast<int64_t>(threadIdx.x) * tiles + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter: tile t writes its digit-d keys from off[d * tiles + t] on,
// in tile order.  The tile is walked in rounds of 256 keys (one per thread,
// in thread order); within a round a key's rank is the keys of the same
// digit in earlier warps plus its rank among its warp's peers.
__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const unsigned long long* keys,
                                                           int64_t count, int shift, int64_t tiles,
                                                           const int64_t* off,
                                                           unsigned long long* out) {
  __shared__ int64_t run[256];                 // next slot of each digit for this tile
  __shared__ uint32_t wc[kRsWarps][256];       // per-warp digit counts of the round
  const int t = threadIdx.x, ln = t & 31, wp = t >> 5;
  run[t] = off[static_cast<int64_t>(t) * tiles + blockIdx.x];
  for (int w = 0; w < kRsWarps; ++w) wc[w][t] = 0u;
  __syncthreads();
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kRsTile;
  for (int r = 0; r < kRsItems; ++r) {
    const int64_t i = base + r * kRsThreads + t;
    const bool ok = i < count;
    const unsigned long long k = ok ? keys[i] : 0ull;
    const int d = ok ? static_cast<int>((k >> shift) & 255ull) : 256;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & ((1u << ln) - 1u));
    if (ok && rank == 0) wc[wp][d] = static_cast<uint32_t>(__popc(peers));
    __syncthreads();
    if (ok) {
      int64_t pos = run[d] + rank;
      for (int w = 0; w < wp; ++w) pos += wc[w][d];
      out[pos] = k;
    }
    __syncthreads();
    uint32_t tot = 0;
    for (int w = 0; w < kRsWarps; ++w) {
      tot += wc[w][t];
      wc[w][t] = 0u;
    }
    run[t] += tot;
    __syncthreads();
  }
}

// ---- scans ---------------------------------------------------------------------
constexpr int kScanThreads = 1024;
constexpr int kScanPer = 4;
constexpr int kScanTileN = kScanThreads * kScanPer;

__device__ __forceinline__ int64_t block_exclusive(int64_t v, int64_t* red, int64_t* total) {
  const int ln = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int64_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (ln >= o) x += y;
  }
  if (ln == 31) red[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int64_t s = red[ln];
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (ln >= o) s += y;
    }
    red[ln] = s;
  }
  __syncthreads();
  const int64_t incl = x + (wid > 0 ? red[wid - 1] : 0);
  *total = red[31];
  __syncthreads();
  return incl - v;
}

// Exclusive scan, phase 1: tile sums.
template <class T>
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(const T* in, int64_t count,
                                                            int64_t* sums) {
  __shared__ int64_t red[32];
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTileN +
                       static_cast<int64_t>(threadIdx.x) * kScanPer;
  int64_t s = 0;
  for (int q = 0; q < kScanPer; ++q)
    if (base + q < count) s += static_cast<int64_t>(in[base + q]);
  int64_t total;
  block_exclusive(s, red, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Phase 2 (one block): exclusive scan of the tile sums in place; *grand = total.
__global__ void __launch_bounds__(kScanThreads) k_scan_sums_excl(int64_t* sums, int64_t tiles,
                                                                 int64_t* grand) {
  __shared__ int64_t red[32];
  int64_t carry = 0;
  for (int64_t b0 = 0; b0 < tiles; b0 += kScanThreads) {
    const int64_t i = b0 + threadIdx.x;
    const int64_t v = i < tiles ? sums[i] : 0;
    int64_t total;
    const int64_t ex = block_exclusive(v, red, &total);
    if (i < tiles) sums[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0 && grand) *grand = carry;
}

// Phase 3: out[i] = exclusive prefix of in.
template <class T>
__global__ void __launch_bounds__(kScanThreads) k_scan_out(const T* in, int64_t count,
                                                           const int64_t* sums, int64_t* out) {
  __shared__ int64_t red[32];
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTileN +
                       static_cast<int64_t>(threadIdx.x) * kScanPer;
  int64_t loc[kScanPer];
  int64_t s = 0;
  for (int q = 0; q < kScanPer; ++q) {
    loc[q] = base + q < count ? static_cast<int64_t>(in[base + q]) : 0;
    s += loc[q];
  }
  int64_t total;
  int64_t run = sums[blockIdx.x] + block_exclusive(s, red, &total);
  for (int q = 0; q < kScanPer; ++q)
    if (base + q < count) {
      out[base + q] = run;
      run += loc[q];
    }
}

// ---- unique arcs and rows --------------------------------------------------------
// keep[i] = 1 for the first copy of each key (sentinels dropped).
__global__ void k_mark_first(const unsigned long long* keys, int64_t count, uint8_t* keep) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const unsigned long long k = keys[i];
    keep[i] = (k != kSentinel && (i == 0 || keys[i - 1] != k)) ? 1 : 0;
  }
}

// colidx[pos[i]] = v and deg[u] += 1 for every kept key.
__global__ void k_emit(const unsigned long long* keys, int64_t count, const uint8_t* keep,
                       const int64_t* pos, int B, int32_t* colidx, unsigned int* deg) {
  const unsigned long long mask = (1ull << B) - 1ull;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (!keep[i]) continue;
    const unsigned long long k = keys[i];
    colidx[pos[i]] = static_cast<int32_t>(k & mask);
    atomicAdd(deg + (k >> B), 1u);
  }
}

// Keys of the kept arcs, compacted (for the in-CSR of a digraph).
__global__ void k_compact_keys(const unsigned long long* keys, int64_t count, const uint8_t* keep,
                               const int64_t* pos, unsigned long long* out) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    if (keep[i]) out[pos[i]] = keys[i];
}

}  // namespace

// ---- host side ----------------------------------------------------------------------
int ingest_bits(int64_t n) {
  int B = 1;
  while ((1ll << B) <= n) ++B;  // ids < n <= 2^B - 1, so no key equals the sentinel
  return B;
}

int64_t scan_tiles(int64_t count) { return (count + kScanTileN - 1) / kScanTileN; }

template <class T>
static int exclusive_scan(cudaStream_t s, const T* in, int64_t count, int64_t* sums, int64_t* out,
                          int64_t* grand) {
  if (count <= 0) return 0;
  const int64_t tiles = scan_tiles(count);
  k_scan_sums<T><<<static_cast<unsigned>(tiles), kScanThreads, 0, s>>>(in, count, sums);
  k_scan_sums_excl<<<1, kScanThreads, 0, s>>>(sums, tiles, grand);
  k_scan_out<T><<<static_cast<unsigned>(tiles), kScanThreads, 0, s>>>(in, count, sums, out);
  return 3;
}

int ingest_make_keys(const LaunchCfg& c, cudaStream_t s, const int32_t* src, const int32_t* dst,
                     int64_t m, int64_t n, int B, int directed, unsigned long long* keys, int* bad) {
  if (m <= 0) return 0;
  k_make_keys<<<c.grid, c.block, 0, s>>>(src, dst, m, n, B, directed, keys, bad);
  return 1;
}

int ingest_swap_keys(const LaunchCfg& c, cudaStream_t s, const unsigned long long* in, int64_t count,
                     int B, unsigned long long* out) {
  if (count <= 0) return 0;
  k_swap_keys<<<c.grid, c.block, 0, s>>>(in, count, B, out);
  return 1;
}

int64_t radix_scratch_words(int64_t count) {
  const int64_t tiles = (count + kRsTile - 1) / kRsTile;
  return 256 * tiles;  // histogram cells; offsets use as many int64 words
}

int radix_sort(cudaStream_t s, unsigned long long*& keys, unsigned long long*& alt, int64_t count,
               int bits, uint32_t* hist, int64_t* off, int64_t* sums) {
  if (count <= 1) return 0;
  const int64_t tiles = (count + kRsTile - 1) / kRsTile;
  int launches = 0;
  for (int shift = 0; shift < bits; shift += 8) {
    k_rs_hist<<<static_cast<unsigned>(tiles), kRsThreads, 0, s>>>(keys, count, shift, tiles, hist);
    launches += 1 + exclusive_scan<uint32_t>(s, hist, 256 * tiles, sums, off, nullptr);
    k_rs_scatter<<<static_cast<unsigned>(tiles), kRsThreads, 0, s>>>(keys, count, shift, tiles, off,
                                                                     alt);
    ++launches;
    unsigned long long* t = keys;
    keys = alt;
    alt = t;
  }
  return launches;
}

int ingest_unique(const LaunchCfg& c, cudaStream_t s, const unsigned long long* keys, int64_t count,
                  uint8_t* keep, int64_t* pos, int64_t* sums, int64_t* nkept) {
  if (count <= 0) return 0;
  k_mark_first<<<c.grid, c.block, 0, s>>>(keys, count, keep);
  return 1 + exclusive_scan<uint8_t>(s, keep, count, sums, pos, nkept);
}

int ingest_emit(const LaunchCfg& c, cudaStream_t s, const unsigned long long* keys, int64_t count,
                const uint8_t* keep, const int64_t* pos, int B, int32_t* colidx, unsigned int* deg) {
  if (count <= 0) return 0;
  k_emit<<<c.grid, c.block, 0, s>>>(keys, count, keep, pos, B, colidx, deg);
  return 1;
}

int ingest_compact(const LaunchCfg& c, cudaStream_t s, const unsigned long long* keys, int64_t count,
                   const uint8_t* keep, const int64_t* pos, unsigned long long* out) {
  if (count <= 0) return 0;
  k_compact_keys<<<c.grid, c.block, 0, s>>>(keys, count, keep, pos, out);
  return 1;
}

int ingest_rowptr(cudaStream_t s, const unsigned int* deg, int64_t n, int64_t* sums,
                  int64_t* rowptr) {
  // rowptr[v] = exclusive prefix of deg, rowptr[n] = total
  return exclusive_scan<unsigned int>(s, deg, n, sums, rowptr, rowptr + n);
}

}  // namespace lgbc
