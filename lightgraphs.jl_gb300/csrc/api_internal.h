// api_internal.h -- shared internals of the C ABI translation units
// (api.cu, api_many.cu, api_learned.cu, api_more.cu): error reporting,
// device allocation, per-handle workspaces, the graph handle itself, and the
// host-side helpers of the level loops that several entry points share.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <utility>
#include <vector>


#include "lgbc.h"
#include "lgbc_kernels.h"

namespace lgbc::api {

using namespace lgbc;

inline thread_local std::string g_last_error;

inline int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

inline int cuda_fail(cudaError_t e, const char* what) {
  return fail(LGBC_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define LGBC_CUDA(call)                                   \
  do {                                                    \
    cudaError_t _e = (call);                              \
    if (_e != cudaSuccess) return cuda_fail(_e, #call);   \
  } while (0)

#define LGBC_TRY(expr)          \
  do {                          \
    int _rc = (expr);           \
    if (_rc != LGBC_OK) return _rc; \
  } while (0)

template <class T>
int dev_alloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return fail(LGBC_ENOMEM, std::string("cudaMalloc of ") + std::to_string(count * sizeof(T)) +
                                 " bytes failed: " + cudaGetErrorString(e));
  }
  return LGBC_OK;
}

template <class T>
void dev_free(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

// Host passes over the vertices of a large graph run on several threads:
// f(part, begin, end) for `parts` contiguous chunks of [0, n), part 0 on the
// calling thread.  Returns the number of parts (1 below 2^16 elements).
template <class F>
int parallel_parts(int64_t n, F&& f) {
  const unsigned hw = std::thread::hardware_concurrency();
  const int parts = n < (int64_t(1) << 16) ? 1 : static_cast<int>(std::max(1u, std::min(8u, hw)));
  std::vector<std::thread> pool;
  for (int p = 1; p < parts; ++p)
    pool.emplace_back([&, p] { f(p, n * p / parts, n * (p + 1) / parts); });
  f(0, int64_t(0), n / parts);
  for (auto& t : pool) t.join();
  return parts;
}

// Multi-source workspace (msbfs.cu): lane sets sized for two words per
// vertex / list entry; path-count and psi rows for `sigma_words` words.
struct MsWorkspace {
  uint64_t* visit = nullptr;
  uint64_t* mb0 = nullptr;
  uint64_t* mb1 = nullptr;
  void* sigma = nullptr;
  void* psi = nullptr;
  int32_t* qv = nullptr;
  uint64_t* qm = nullptr;
  unsigned long long* lvl_off = nullptr;
  BatchCtl* ctl = nullptr;
  unsigned* claim = nullptr;    // two-word batches only
  unsigned long long cap = 0;
  int sigma_words = 0;          // 0: no path-count rows yet

  void release() {
    dev_free(visit);
    dev_free(mb0);
    dev_free(mb1);
    if (sigma) cudaFree(sigma);
    if (psi) cudaFree(psi);
    sigma = psi = nullptr;
    dev_free(qv);
    dev_free(qm);
    dev_free(lvl_off);
    dev_free(ctl);
    dev_free(claim);
    cap = 0;
    sigma_words = 0;
  }
};

// Hub work items (see HubItem in lgbc_kernels.h) and their accumulators.
struct HubTable {
  HubItem* out_items = nullptr;
  int64_t n_out = 0;
  HubItem* in_items = nullptr;   // == out_items for undirected graphs
  int64_t n_in = 0;
  unsigned long long* acc = nullptr;
  unsigned long long* mask = nullptr;
  unsigned int* cnt = nullptr;
  int64_t nslots = 0;
  int built_for = -1;            // hub_degree the table was built with
  int built_order = -1;          // and hub_order
  void release() {
    if (in_items && in_items != out_items) cudaFree(in_items);
    dev_free(out_items);
    in_items = nullptr;
    dev_free(acc);
    dev_free(mask);
    dev_free(cnt);
    n_out = n_in = nslots = 0;
    built_for = -1;
    built_order = -1;
  }
};

struct BfsWorkspace {
  int32_t* queue = nullptr;
  uint32_t* bm0 = nullptr;
  uint32_t* bm1 = nullptr;
  BatchCtl* ctl = nullptr;
  int32_t* large = nullptr;
  void release() {
    dev_free(large);
    dev_free(queue);
    dev_free(bm0);
    dev_free(bm1);
    dev_free(ctl);
  }
};

// Learned-proposal state of a graph (learned.cu): core numbers, features,
// scores, the proposal p and its CDF, and scan scratch.
struct LearnedWorkspace {
  int32_t* core = nullptr;
  uint8_t* flag = nullptr;
  int32_t* list = nullptr;
  int32_t* large = nullptr;                // hubs deferred by a core pass
  int32_t* log_v = nullptr;                // vertices lowered by a core pass
  int32_t* log_old = nullptr;              //   and their values before it
  int32_t* hub_v = nullptr;                // the same for the hubs
  int32_t* hub_old = nullptr;
  unsigned long long* counters = nullptr;  // [0] self-loop flag, [1] lowered this pass,
                                           // [2] list size, [3] deferred hubs, [4] lowered hubs
  float4* feat = nullptr;
  float* y = nullptr;
  float* fscr = nullptr;
  double* e = nullptr;
  double* tsum = nullptr;
  double* scal = nullptr;
  double* p = nullptr;
  double* cdf = nullptr;
  int32_t* samp = nullptr;
  double* samp_w = nullptr;
  int64_t samp_cap = 0;
  bool built = false;
  int64_t core_passes = 0;
  void release() {
    dev_free(core);
    dev_free(flag);
    dev_free(list);
    dev_free(large);
    dev_free(log_v);
    dev_free(log_old);
    dev_free(hub_v);
    dev_free(hub_old);
    dev_free(counters);
    dev_free(feat);
    dev_free(y);
    dev_free(fscr);
    dev_free(e);
    dev_free(tsum);
    dev_free(scal);
    dev_free(p);
    dev_free(cdf);
    dev_free(samp);
    dev_free(samp_w);
    samp_cap = 0;
    built = false;
  }
};

// A device-driven level loop instantiated for one configuration.
struct LoopKey {
  int backward;                 // 0 forward sweep, 1 backward (dependency) sweep
  int sigma_kind;
  LaneSet act;
  const int32_t* dist;
  int64_t dist_ld;
  const double* bc;
  MsBuffers b;                  // lane_src and lane_w zeroed: not used inside the loop
  HubData hd;
  double alpha, beta;
};
struct LoopGraph {
  LoopKey key;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int td_kernels = 0;           // kernels per top-down / bottom-up / backward level
  int bu_kernels = 0;
  int body_kernels = 0;
  uint64_t last_use = 0;
  void release() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
  }
};

}  // namespace lgbc::api

namespace lgbc::api {
// Explicit (vertex, lane mask) seeds on the device, for unions of graphs;
// the vertices are distinct (a vertex that starts several lanes has them all
// in its mask).
struct Seeds {
  const int32_t* v = nullptr;
  const uint64_t* mask = nullptr;   // one lane set per seed (1 or 2 words: the batch's)
  int64_t count = 0;
  // optional premark of seedless lanes per component (unions of graphs)
  const int64_t* seg_off = nullptr;
  const uint64_t* seg_mark = nullptr;  // one lane set per component
  int64_t nseg = 0;
  // stacked unions with lane weights: one row of 64 * words weights per copy
  // of an lane_w_n-vertex graph, lane_w_count weights in all
  int64_t lane_w_n = 0;
  int64_t lane_w_count = 0;
};
// Forward-sweep export of a one-word batch with path counts (lgbc_path_counts):
// the batch stops after its forward sweep, with sigma / dist written per lane.
struct PathExport {
  double* sigma = nullptr;
  int32_t* dist = nullptr;  // may be null
  int64_t ld = 0;           // row length (n)
};
}  // namespace lgbc::api

struct lgbc_graph {
  int device = 0;
  int64_t n = 0;
  int64_t nnz = 0;
  int directed = 0;
  cudaStream_t stream = nullptr;
  int64_t* d_rowptr = nullptr;
  int32_t* d_colidx = nullptr;
  int64_t* d_in_rowptr = nullptr;   // == d_rowptr for undirected graphs
  int32_t* d_in_colidx = nullptr;
  std::vector<uint8_t> has_degree;  // degree(g, v) > 0, host copy for filtering
  std::mutex mu;
  lgbc::api::MsWorkspace ms;
  lgbc::api::BfsWorkspace bfs;
  lgbc::api::HubTable hubs;
  lgbc::api::LearnedWorkspace learned;
  int32_t* d_src = nullptr;         // device copy of a call's source list
  int64_t d_src_cap = 0;
  double* d_bc = nullptr;           // device result buffer for host-buffer calls
  int32_t* d_dist = nullptr;        // device distance buffer (gdistances)
  int64_t d_dist_cap = 0;
  lgbc::BatchCtl* h_ctl = nullptr;        // pinned mirror of a control block
  cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
  int64_t launches = 0;             // running count of kernels launched
  int64_t launches_at_start = 0;
  lgbc::LaunchCfg cfg{};
  size_t max_smem = 0;
  unsigned long long sigma_limit = ~0ull;  // (2^64 - 1) / (max in-degree + 1)
  lgbc_stats stats{};
  lgbc_tuning tune{14.0, 24.0, 256, 128, 32, 0, 1, 1, 1 << 21, 2, 0};
  lgbc_graph* stack = nullptr;        // R copies of this graph (stacked batches)
  int64_t stack_copies = 0;
  std::vector<int32_t> h_active;      // the last call's ordered active sources
  std::vector<double> h_weights;      // their weights (weighted calls; empty otherwise)
  double* d_lw_fixed = nullptr;       // lane weights of the running batch (cached graphs)
  int64_t d_lw_cap = 0;
  cudaStream_t cap_stream = nullptr;  // stream used to capture level-loop graphs
  std::vector<lgbc::api::LoopGraph> loops;       // cached device-driven level loops
  uint64_t loop_clock = 0;
  std::vector<int32_t> landmarks;   // the highest-degree vertices (source ordering)
  int32_t* d_lmdist = nullptr;      // landmarks x n BFS distances, computed on first use

  lgbc::DevGraph dev() const {
    return lgbc::DevGraph{n, nnz, d_rowptr, d_colidx, d_in_rowptr, d_in_colidx};
  }
};

namespace lgbc::api {

// Helpers shared by the entry points (api.cu).
int check_graph(const lgbc_graph* g);
int use_device(lgbc_graph* g);
int check_sources(const lgbc_graph* g, const int32_t* src, int64_t nsrc);
int ensure_src(lgbc_graph* g, int64_t count);
// Multi-source workspace; with need_sigma, path-count / psi rows for batches
// of up to 64 * words lanes.
int ensure_ms(lgbc_graph* g, bool need_sigma, int words = 1);
int ensure_bfs(lgbc_graph* g);
int ensure_dist(lgbc_graph* g, int64_t count);
int ensure_hubs(lgbc_graph* g);
HubData hub_data(const lgbc_graph* g);
int read_ctl(lgbc_graph* g, const BatchCtl* dctl);
int check_launch(lgbc_graph* g);
MsBuffers ms_buffers(lgbc_graph* g, const int32_t* lane_src, const double* lane_w = nullptr);
// One multi-source batch: forward level loop, then (with sigma) the backward
// dependency sweep into bc.  Returns LGBC_OK, or 1 when the batch must be
// replayed with FP64 path counts.  lane_w (sigma batches): per-lane weights of
// the accumulation into bc; stats (distance-only batches): per-lane distance
// statistics, accumulated; stress (distance-only batches): the stress sweep;
// pexp (one-word batches with path counts): export the forward sweep and
// skip the dependency sweep.
int run_ms_batch(lgbc_graph* g, const int32_t* lane_src, int nl, int sigma_kind, double* bc,
                 int32_t* dist, int64_t dist_ld, const Seeds& seeds = Seeds(),
                 const double* lane_w = nullptr, const LevelStats* stats = nullptr,
                 unsigned long long* stress = nullptr, const PathExport* pexp = nullptr);
// The path-count / dependency kind of a Brandes batch on this handle: exact
// uint64 path counts with FP64 dependencies (default) or, with the
// dependency_df32 tuning field, double-float dependencies.
inline int dep_kind(const lgbc_graph* g) {
  return g->tune.dependency_df32 ? kSigmaU64 : kSigmaU64F64;
}
// Brandes over the active sources already on the device (g->d_src[0, k)),
// accumulating into bc_dev (zeroed here); with d_w, source i's dependencies
// are scaled by d_w[i].
int run_betweenness(lgbc_graph* g, int64_t k_act, int endpoints, double* bc_dev,
                    const double* d_w = nullptr);
int order_active(lgbc_graph* g, std::vector<int32_t>& act, std::vector<double>* w);
int prepare_sources(lgbc_graph* g, const int32_t* src, int64_t nsrc, int64_t* k_act);
void reset_stats(lgbc_graph* g);
void finish_stats(lgbc_graph* g);
int init_handle(lgbc_graph* g, int64_t n, int directed);
// Host rowptr copies are required; colidx copies may be null (copied back
// from the device when the hub items need them).
int finish_handle(lgbc_graph* g, const int64_t* rowptr, const int64_t* in_rowptr,
                  const int32_t* colidx = nullptr, const int32_t* in_colidx = nullptr);
int run_bfs(lgbc_graph* g, const DevGraph& dg, int64_t nsrc);
int prepare_bfs(lgbc_graph* g, const int32_t* src, int64_t nsrc);

}  // namespace lgbc::api
