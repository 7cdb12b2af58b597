// noalloc.cu -- gdistances for callers that cannot allocate device memory.
//
// lgbc_gdistances needs a graph handle, whose CSR and BFS workspace come from
// cudaMalloc.  Some callers cannot allocate: hosts whose device memory
// belongs to another allocator with a fixed budget (a Julia CuArray pool, a
// serving process that reserves the GPU's memory when it starts), where an
// outside cudaMalloc can fail or take memory the budget counts on, and loops
// that must not pay the device-wide synchronisation of cudaFree.
// lgbc_gdistances_noalloc takes every input and output as caller-owned device
// pointers and keeps its own scratch -- the frontier queue, the two frontier
// bitmaps, the level control block and the input-check flag -- in the
// file-scope device array below, which every GPU that loads the library holds
// until the process exits.  Its size fixes the largest graph:
// LGBC_NOALLOC_MAX_VERTICES vertices.  Each call clears what must start at
// zero (the check flag here; bitmaps and control block in bfs_init), and
// calls that overlap on the GPU race on the shared array.
#include <cstdio>
#include <mutex>

#include "lgbc.h"
#include "lgbc_kernels.h"

namespace lgbc {
namespace {

constexpr int64_t kMaxN = LGBC_NOALLOC_MAX_VERTICES;
constexpr size_t kAlign = 256;
constexpr size_t round_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }
constexpr int64_t kWords = (kMaxN + 31) / 32 + 4;  // +4: room for 16-byte staging copies
constexpr size_t kCtlOff = 0;
constexpr size_t kBadOff = round_up(sizeof(BatchCtl));
constexpr size_t kBm0Off = kBadOff + kAlign;
constexpr size_t kBm1Off = kBm0Off + round_up(static_cast<size_t>(kWords) * 4);
constexpr size_t kQueueOff = kBm1Off + round_up(static_cast<size_t>(kWords) * 4);
constexpr size_t kScratchBytes = kQueueOff + round_up(static_cast<size_t>(kMaxN + 1) * 4);

// The scratch: control block, error flag, two bitmaps, the level queue.
// Shared by every call on a device; each call clears what must start at zero.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Host-side view of each device's scratch address (set once per device).
struct DeviceSetup {
  unsigned char* base = nullptr;
  LaunchCfg cfg{};
  size_t max_smem = 0;
};
std::mutex g_setup_mu;
DeviceSetup g_setup[256];

// Sets bit 0 of *bad when a source id is outside [0, n).
__global__ void k_check_sources(const int32_t* src, int64_t nsrc, int64_t n, int* bad) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < nsrc;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    if (src[i] < 0 || src[i] >= n) atomicOr(bad, 1);
}

int err(int code, const char* msg) {
  set_last_error(msg);
  return code;
}

int cuda_err(cudaError_t e, const char* what) {
  static thread_local char buf[256];
  snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  return err(LGBC_ECUDA, buf);
}

#define NA_CUDA(call)                                  \
  do {                                                 \
    cudaError_t _e = (call);                           \
    if (_e != cudaSuccess) return cuda_err(_e, #call); \
  } while (0)

// Once per device, with that device current: look up the scratch address
// (cudaGetSymbolAddress) and the launch shape.
int setup_device(int dev, DeviceSetup** out) {
  if (dev < 0 || dev >= 256) return err(LGBC_ECUDA, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_setup_mu);
  DeviceSetup& s = g_setup[dev];
  if (!s.base) {
    void* p = nullptr;
    NA_CUDA(cudaGetSymbolAddress(&p, g_scratch));
    int sms = 0;
    NA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int smem = 0;
    NA_CUDA(cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    bfs_configure(static_cast<size_t>(smem));
    s.cfg = LaunchCfg{sms * 8, 256, sms};
    s.max_smem = static_cast<size_t>(smem);
    s.base = static_cast<unsigned char*>(p);
  }
  *out = &s;
  return LGBC_OK;
}

}  // namespace
}  // namespace lgbc

using namespace lgbc;

extern "C" int lgbc_gdistances_noalloc(int64_t n, int64_t nnz, const int64_t* rowptr,
                                       const int32_t* colidx, const int64_t* in_rowptr,
                                       const int32_t* in_colidx, const int32_t* src, int64_t nsrc,
                                       int32_t* dist, void* stream) {
  if (n < 0 || nnz < 0 || nsrc < 0) return err(LGBC_EINVAL, "negative size");
  if (n > kMaxN)
    return err(LGBC_EINVAL,
               "lgbc_gdistances_noalloc: the graph has more vertices than the fixed scratch holds "
               "(LGBC_NOALLOC_MAX_VERTICES); use lgbc_graph_create + lgbc_gdistances");
  if (n == 0) return LGBC_OK;
  if (!rowptr || (nnz > 0 && !colidx) || !dist || (nsrc > 0 && !src))
    return err(LGBC_EINVAL, "null device pointer");
  if ((in_rowptr && nnz > 0 && !in_colidx) || (!in_rowptr && in_colidx))
    return err(LGBC_EINVAL, "pass both in_rowptr and in_colidx (directed) or neither");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0;
  NA_CUDA(cudaGetDevice(&dev));
  DeviceSetup* ds = nullptr;
  const int rc = setup_device(dev, &ds);
  if (rc != LGBC_OK) return rc;

  BatchCtl* ctl = reinterpret_cast<BatchCtl*>(ds->base + kCtlOff);
  int* bad = reinterpret_cast<int*>(ds->base + kBadOff);
  BfsBuffers b{reinterpret_cast<int32_t*>(ds->base + kQueueOff),
               {reinterpret_cast<uint32_t*>(ds->base + kBm0Off),
                reinterpret_cast<uint32_t*>(ds->base + kBm1Off)},
               ctl};
  const bool directed = in_rowptr != nullptr;
  const DevGraph g{n, nnz, rowptr, colidx, directed ? in_rowptr : rowptr,
                   directed ? in_colidx : colidx};
  const LaunchCfg& c = ds->cfg;

  // inputs are checked on the device before anything indexes with them
  NA_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), s));
  validate_csr(c, s, g.rowptr, g.colidx, n, nnz, bad);
  if (directed) validate_csr(c, s, g.in_rowptr, g.in_colidx, n, nnz, bad);
  if (nsrc > 0) k_check_sources<<<c.grid, c.block, 0, s>>>(src, nsrc, n, bad);
  NA_CUDA(cudaGetLastError());
  int h_bad = 0;
  NA_CUDA(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  NA_CUDA(cudaStreamSynchronize(s));
  if (h_bad)
    return err(LGBC_EINVAL,
               "lgbc_gdistances_noalloc: invalid CSR (rowptr must run from 0 to nnz without "
               "decreasing, column ids in [0, n)) or a source id outside [0, n)");

  // the same level loop as lgbc_gdistances (bfs.cu kernels), default tuning
  const double alpha = 14.0, beta = 24.0;
  fill_i32(c, s, dist, n, kUnreached);
  bfs_init(c, s, g, b, src, nsrc, dist);
  NA_CUDA(cudaGetLastError());
  BatchCtl h{};
  NA_CUDA(cudaMemcpyAsync(&h, ctl, sizeof(BatchCtl), cudaMemcpyDeviceToHost, s));
  NA_CUDA(cudaStreamSynchronize(s));
  const size_t bm_bytes = static_cast<size_t>(((n + 31) / 32 + 3) & ~int64_t(3)) * 4;
  const int stage = bm_bytes <= ds->max_smem ? 1 : 0;
  bool bu = false;
  int64_t levels = 0;
  while (!h.done) {
    const double mf = static_cast<double>(h.mf_cur);
    const double mu = static_cast<double>(nnz) - static_cast<double>(h.mu_done);
    const double nf = static_cast<double>(h.hi - h.lo);
    bu = bu ? (nf >= static_cast<double>(n) / beta) : (mf > mu / alpha);
    if (bu) bfs_bottomup(c, s, g, b, dist, stage);
    else bfs_topdown(c, s, g, b, dist);
    bfs_advance(s, b);
    NA_CUDA(cudaGetLastError());
    NA_CUDA(cudaMemcpyAsync(&h, ctl, sizeof(BatchCtl), cudaMemcpyDeviceToHost, s));
    NA_CUDA(cudaStreamSynchronize(s));
    if (++levels > n + 1) return err(LGBC_ETIMEOUT, "BFS exceeded n + 1 levels");
  }
  return LGBC_OK;
}
