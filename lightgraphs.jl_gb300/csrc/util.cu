// util.cu -- fills and the endpoint terms of the betweenness accumulation.
#include "lgbc_kernels.h"

namespace lgbc {
namespace {

template <class T>
__global__ void k_fill(T* p, int64_t count, T value) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    p[i] = value;
}

// _accumulate_endpoints! (src/centrality/betweenness.jl:109-134) adds, per
// source s, length(S) - 1 = n - 1 to betweenness[s] (:122; S always holds all
// n vertices, dijkstra.jl:126-132) and 1 to every other vertex (:130).  Summed
// over the active sources: k_act to every vertex, then n - 2 more to each
// source occurrence.
__global__ void k_add_all(double* bc, int64_t n, double k) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    bc[i] += k;
}

__global__ void k_add_sources(double* bc, const int32_t* src, int64_t k, double extra) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < k;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    atomicAdd(bc + src[i], extra);
}

// Flags (bit 0) a decreasing rowptr step, (bit 1) a column index outside
// [0, n) and (bit 2) a rowptr that does not start at 0 or end at nnz; the
// host rejects the graph when any bit is set.  With all three clear every row
// range lies inside [0, nnz), so no kernel indexes colidx out of bounds.
__global__ void k_validate_csr(const int64_t* rowptr, const int32_t* colidx, int64_t n, int64_t nnz,
                               int* bad) {
  int local = 0;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  if (blockIdx.x == 0 && threadIdx.x == 0 && (rowptr[0] != 0 || rowptr[n] != nnz)) local |= 4;
  for (int64_t v = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; v < n; v += stride)
    if (rowptr[v + 1] < rowptr[v]) local |= 1;
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < nnz; e += stride) {
    const int32_t c = colidx[e];
    if (c < 0 || c >= n) local |= 2;
  }
  if (__any_sync(kFull, local != 0) && local) atomicOr(bad, local);
}

__global__ void k_add_segments(double* bc, const int64_t* seg_off, const double* seg_add,
                               int64_t nseg) {
  for (int64_t sgi = blockIdx.x; sgi < nseg; sgi += gridDim.x) {
    const double a = seg_add[sgi];
    if (a == 0.0) continue;
    for (int64_t v = seg_off[sgi] + threadIdx.x; v < seg_off[sgi + 1]; v += blockDim.x) bc[v] += a;
  }
}

__global__ void k_add_sources_var(double* bc, const int32_t* src, const double* add, int64_t k) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < k;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    atomicAdd(bc + src[i], add[i]);
}

}  // namespace

int add_endpoints_many(const LaunchCfg& c, cudaStream_t s, double* bc, const int64_t* seg_off,
                       const double* seg_add, int64_t nseg, const int32_t* src,
                       const double* src_add, int64_t nsrc) {
  int launches = 0;
  if (nseg > 0) {
    k_add_segments<<<c.grid, c.block, 0, s>>>(bc, seg_off, seg_add, nseg);
    ++launches;
  }
  if (nsrc > 0) {
    k_add_sources_var<<<c.grid, c.block, 0, s>>>(bc, src, src_add, nsrc);
    ++launches;
  }
  return launches;
}

int validate_csr(const LaunchCfg& c, cudaStream_t s, const int64_t* rowptr, const int32_t* colidx,
                 int64_t n, int64_t nnz, int* bad) {
  k_validate_csr<<<c.grid, c.block, 0, s>>>(rowptr, colidx, n, nnz, bad);
  return 1;
}

namespace {
__global__ void k_gather_cols(const int32_t* dist, int64_t ld, int nl, const int32_t* src,
                              int64_t k, int32_t* out) {
  const int64_t total = k * nl;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t r = i / nl;
    const int j = static_cast<int>(i - r * nl);
    out[i] = dist[static_cast<int64_t>(j) * ld + src[r]];
  }
}
}  // namespace

int gather_cols(const LaunchCfg& c, cudaStream_t s, const int32_t* dist, int64_t ld, int nl,
                const int32_t* src, int64_t k, int32_t* out) {
  if (k <= 0 || nl <= 0) return 0;
  k_gather_cols<<<c.grid, c.block, 0, s>>>(dist, ld, nl, src, k, out);
  return 1;
}

namespace {
__global__ void k_sum_copies(const double* stacked, int64_t n, int64_t copies, double* out) {
  for (int64_t v = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; v < n;
       v += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double acc = 0.0;
    for (int64_t r = 0; r < copies; ++r) acc += stacked[r * n + v];
    out[v] = acc;
  }
}
// Disjoint union of `copies` copies of a CSR: copy r holds vertices
// [r n, (r + 1) n) and entries [r nnz, (r + 1) nnz).  rp1 has copies n + 1
// entries (index copies n reads rp0[0] = 0, giving copies nnz).
__global__ void k_replicate_rows(const int64_t* rp0, int64_t n, int64_t nnz, int64_t copies,
                                 int64_t* rp1) {
  const int64_t total = copies * n + 1;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t r = i / n;
    rp1[i] = r * nnz + rp0[i - r * n];
  }
}

__global__ void k_replicate_cols(const int32_t* c0, int64_t nnz, int64_t n, int64_t copies,
                                 int32_t* c1) {
  const int64_t total = copies * nnz;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t r = i / nnz;
    c1[i] = static_cast<int32_t>(r * n + c0[i - r * nnz]);
  }
}
}  // namespace

int replicate_csr(const LaunchCfg& c, cudaStream_t s, const int64_t* rp0, const int32_t* c0,
                  int64_t n, int64_t nnz, int64_t copies, int64_t* rp1, int32_t* c1) {
  if (n <= 0 || copies <= 0) return 0;
  k_replicate_rows<<<c.grid, c.block, 0, s>>>(rp0, n, nnz, copies, rp1);
  if (nnz <= 0) return 1;
  k_replicate_cols<<<c.grid, c.block, 0, s>>>(c0, nnz, n, copies, c1);
  return 2;
}

int sum_copies(const LaunchCfg& c, cudaStream_t s, const double* stacked, int64_t n, int64_t copies,
               double* out) {
  if (n <= 0) return 0;
  k_sum_copies<<<c.grid, c.block, 0, s>>>(stacked, n, copies, out);
  return 1;
}

int fill_i32(const LaunchCfg& c, cudaStream_t s, int32_t* p, int64_t count, int32_t value) {
  if (count <= 0) return 0;
  k_fill<int32_t><<<c.grid, c.block, 0, s>>>(p, count, value);
  return 1;
}

int fill_f64(const LaunchCfg& c, cudaStream_t s, double* p, int64_t count, double value) {
  if (count <= 0) return 0;
  k_fill<double><<<c.grid, c.block, 0, s>>>(p, count, value);
  return 1;
}

int add_endpoints(const LaunchCfg& c, cudaStream_t s, double* bc, int64_t n,
                  const int32_t* active_src, int64_t k_act) {
  if (k_act <= 0 || n <= 0) return 0;
  k_add_all<<<c.grid, c.block, 0, s>>>(bc, n, static_cast<double>(k_act));
  k_add_sources<<<c.grid, c.block, 0, s>>>(bc, active_src, k_act, static_cast<double>(n) - 2.0);
  return 2;
}

}  // namespace lgbc
