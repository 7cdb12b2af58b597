// api.cu -- the C ABI of include/lgbc.h: graph handles, workspaces and the
// host side of the level loops.  All arithmetic runs in the kernels of
// msbfs.cu / bfs.cu / util.cu; there is no CPU fallback.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "lgbc.h"
#include "lgbc_kernels.h"

using namespace lgbc;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
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

// Multi-source workspace (msbfs.cu), sized for one batch of 64 lanes.
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
  unsigned long long cap = 0;
  bool have_sigma = false;

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
    cap = 0;
    have_sigma = false;
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
  void release() {
    if (in_items && in_items != out_items) cudaFree(in_items);
    dev_free(out_items);
    in_items = nullptr;
    dev_free(acc);
    dev_free(mask);
    dev_free(cnt);
    n_out = n_in = nslots = 0;
    built_for = -1;
  }
};

struct BfsWorkspace {
  int32_t* queue = nullptr;
  uint32_t* bm0 = nullptr;
  uint32_t* bm1 = nullptr;
  BatchCtl* ctl = nullptr;
  void release() {
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
  unsigned long long* counters = nullptr;  // [0] self-loop flag, [1] lowered, [2] list size
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
  unsigned long long act;
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

}  // namespace

// Lets the other translation units of the library report errors through
// lgbc_last_error().
void lgbc::set_last_error(const char* msg) { g_last_error = msg ? msg : ""; }

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
  MsWorkspace ms;
  BfsWorkspace bfs;
  HubTable hubs;
  LearnedWorkspace learned;
  int32_t* d_src = nullptr;         // device copy of a call's source list
  int64_t d_src_cap = 0;
  double* d_bc = nullptr;           // device result buffer for host-buffer calls
  int32_t* d_dist = nullptr;        // device distance buffer (gdistances)
  int64_t d_dist_cap = 0;
  BatchCtl* h_ctl = nullptr;        // pinned mirror of a control block
  cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
  int64_t launches = 0;             // running count of kernels launched
  int64_t launches_at_start = 0;
  LaunchCfg cfg{};
  size_t max_smem = 0;
  unsigned long long sigma_limit = ~0ull;  // (2^64 - 1) / (max in-degree + 1)
  lgbc_stats stats{};
  lgbc_tuning tune{14.0, 24.0, 256, 64, 32, 0, 1, 1, 1 << 21, 0};
  lgbc_graph* stack = nullptr;        // R copies of this graph (stacked batches)
  int64_t stack_copies = 0;
  std::vector<int32_t> h_active;      // the last call's ordered active sources
  std::vector<double> h_weights;      // their weights (weighted calls; empty otherwise)
  double* d_lw_fixed = nullptr;       // lane weights of the running batch (cached graphs)
  int64_t d_lw_cap = 0;
  cudaStream_t cap_stream = nullptr;  // stream used to capture level-loop graphs
  std::vector<LoopGraph> loops;       // cached device-driven level loops
  uint64_t loop_clock = 0;
  std::vector<int32_t> landmarks;   // the highest-degree vertices (source ordering)
  int32_t* d_lmdist = nullptr;      // landmarks x n BFS distances, computed on first use

  DevGraph dev() const {
    return DevGraph{n, nnz, d_rowptr, d_colidx, d_in_rowptr, d_in_colidx};
  }
};

namespace {

int check_graph(const lgbc_graph* g) {
  if (!g) return fail(LGBC_EINVAL, "null graph handle");
  return LGBC_OK;
}

int use_device(lgbc_graph* g) {
  LGBC_CUDA(cudaSetDevice(g->device));
  return LGBC_OK;
}

int check_sources(const lgbc_graph* g, const int32_t* src, int64_t nsrc) {
  if (nsrc < 0) return fail(LGBC_EINVAL, "negative source count");
  if (nsrc > 0 && !src) return fail(LGBC_EINVAL, "null source list");
  for (int64_t i = 0; i < nsrc; ++i) {
    if (src[i] < 0 || src[i] >= g->n) {
      char buf[160];
      std::snprintf(buf, sizeof buf, "source %lld at position %lld is not a vertex of a graph with %lld vertices",
                    static_cast<long long>(src[i]), static_cast<long long>(i),
                    static_cast<long long>(g->n));
      return fail(LGBC_EINVAL, buf);
    }
  }
  return LGBC_OK;
}

int ensure_src(lgbc_graph* g, int64_t count) {
  if (count <= g->d_src_cap) return LGBC_OK;
  dev_free(g->d_src);
  g->d_src_cap = 0;
  LGBC_TRY(dev_alloc(&g->d_src, static_cast<size_t>(std::max<int64_t>(count, 64))));
  g->d_src_cap = std::max<int64_t>(count, 64);
  return LGBC_OK;
}

int ensure_ms(lgbc_graph* g, bool need_sigma) {
  MsWorkspace& w = g->ms;
  const size_t n = static_cast<size_t>(g->n);
  if (!w.visit) {
    LGBC_TRY(dev_alloc(&w.visit, n));
    LGBC_TRY(dev_alloc(&w.mb0, n));
    LGBC_TRY(dev_alloc(&w.mb1, n));
    LGBC_TRY(dev_alloc(&w.lvl_off, n + 3));
    LGBC_TRY(dev_alloc(&w.ctl, 1));
    LGBC_CUDA(cudaMemsetAsync(w.visit, 0, n * 8, g->stream));
    LGBC_CUDA(cudaMemsetAsync(w.mb0, 0, n * 8, g->stream));
    LGBC_CUDA(cudaMemsetAsync(w.mb1, 0, n * 8, g->stream));
  }
  if (!w.qv) {
    const unsigned long long cap = 4ull * n + 1024;
    LGBC_TRY(dev_alloc(&w.qv, cap));
    LGBC_TRY(dev_alloc(&w.qm, cap));
    w.cap = cap;
  }
  if (need_sigma && !w.have_sigma) {
    unsigned long long* s = nullptr;
    unsigned long long* p = nullptr;
    LGBC_TRY(dev_alloc(&s, n * kMaxLanes));
    int rc = dev_alloc(&p, n * kMaxLanes);
    if (rc != LGBC_OK) {
      cudaFree(s);
      return rc;
    }
    w.sigma = s;
    w.psi = p;
    w.have_sigma = true;
  }
  return LGBC_OK;
}

int grow_ms_lists(lgbc_graph* g) {
  MsWorkspace& w = g->ms;
  const unsigned long long n = static_cast<unsigned long long>(g->n);
  const unsigned long long max_cap = 65ull * n + 1024;  // 64 lanes x n levels + level 0
  unsigned long long cap = std::min(max_cap, w.cap * 2);
  if (cap <= w.cap) return fail(LGBC_ENOMEM, "level lists cannot grow further");
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  dev_free(w.qv);
  dev_free(w.qm);
  LGBC_TRY(dev_alloc(&w.qv, cap));
  LGBC_TRY(dev_alloc(&w.qm, cap));
  w.cap = cap;
  return LGBC_OK;
}

int ensure_bfs(lgbc_graph* g) {
  BfsWorkspace& w = g->bfs;
  if (w.queue) return LGBC_OK;
  const size_t n = static_cast<size_t>(g->n);
  const size_t words = (n + 31) / 32 + 4;
  LGBC_TRY(dev_alloc(&w.queue, n + 1));
  LGBC_TRY(dev_alloc(&w.bm0, words));
  LGBC_TRY(dev_alloc(&w.bm1, words));
  LGBC_TRY(dev_alloc(&w.ctl, 1));
  return LGBC_OK;
}

int ensure_dist(lgbc_graph* g, int64_t count) {
  if (count <= g->d_dist_cap) return LGBC_OK;
  dev_free(g->d_dist);
  g->d_dist_cap = 0;
  LGBC_TRY(dev_alloc(&g->d_dist, static_cast<size_t>(count)));
  g->d_dist_cap = count;
  return LGBC_OK;
}

// Cut every edge list longer than H into kHubChunk-edge items.
void make_items(const int64_t* rowptr, int64_t n, int H, const std::vector<int32_t>& slot_of,
                std::vector<HubItem>& items) {
  items.clear();
  for (int64_t v = 0; v < n; ++v) {
    const int64_t e0 = rowptr[v], e1 = rowptr[v + 1];
    if (e1 - e0 <= H) continue;
    const int32_t nit = static_cast<int32_t>((e1 - e0 + kHubChunk - 1) / kHubChunk);
    for (int64_t lo = e0; lo < e1; lo += kHubChunk) {
      HubItem it;
      it.lo = lo;
      it.hi = std::min<int64_t>(lo + kHubChunk, e1);
      it.v = static_cast<int32_t>(v);
      it.slot = slot_of[static_cast<size_t>(v)];
      it.nitems = nit;
      it.pad = 0;
      items.push_back(it);
    }
  }
}

int upload_items(const std::vector<HubItem>& items, HubItem** out) {
  *out = nullptr;
  if (items.empty()) return LGBC_OK;
  LGBC_TRY(dev_alloc(out, items.size()));
  LGBC_CUDA(cudaMemcpy(*out, items.data(), items.size() * sizeof(HubItem), cudaMemcpyHostToDevice));
  return LGBC_OK;
}

// Build the hub work items from host copies of rowptr / in_rowptr.
int build_hubs(lgbc_graph* g, const int64_t* rowptr, const int64_t* in_rowptr, int H) {
  g->hubs.release();
  const int64_t n = g->n;
  std::vector<int32_t> slot_of(static_cast<size_t>(n), -1);
  int64_t nslots = 0;
  for (int64_t v = 0; v < n; ++v) {
    const int64_t dout = rowptr[v + 1] - rowptr[v];
    const int64_t din = in_rowptr[v + 1] - in_rowptr[v];
    if (dout > H || din > H) slot_of[static_cast<size_t>(v)] = static_cast<int32_t>(nslots++);
  }
  g->hubs.nslots = nslots;
  g->hubs.built_for = H;
  if (nslots == 0) return LGBC_OK;
  std::vector<HubItem> items;
  make_items(rowptr, n, H, slot_of, items);
  g->hubs.n_out = static_cast<int64_t>(items.size());
  LGBC_TRY(upload_items(items, &g->hubs.out_items));
  if (g->directed) {
    make_items(in_rowptr, n, H, slot_of, items);
    g->hubs.n_in = static_cast<int64_t>(items.size());
    LGBC_TRY(upload_items(items, &g->hubs.in_items));
  } else {
    g->hubs.in_items = g->hubs.out_items;
    g->hubs.n_in = g->hubs.n_out;
  }
  LGBC_TRY(dev_alloc(&g->hubs.acc, static_cast<size_t>(nslots) * kMaxLanes));
  LGBC_TRY(dev_alloc(&g->hubs.mask, static_cast<size_t>(nslots)));
  LGBC_TRY(dev_alloc(&g->hubs.cnt, static_cast<size_t>(nslots)));
  LGBC_CUDA(cudaMemset(g->hubs.acc, 0, static_cast<size_t>(nslots) * kMaxLanes * 8));
  LGBC_CUDA(cudaMemset(g->hubs.mask, 0, static_cast<size_t>(nslots) * 8));
  LGBC_CUDA(cudaMemset(g->hubs.cnt, 0, static_cast<size_t>(nslots) * 4));
  return LGBC_OK;
}

// Rebuild the hub table after hub_degree changed (rowptr copied back).
int ensure_hubs(lgbc_graph* g) {
  if (g->hubs.built_for == g->tune.hub_degree) return LGBC_OK;
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  std::vector<int64_t> rp(static_cast<size_t>(g->n + 1)), irp;
  LGBC_CUDA(cudaMemcpy(rp.data(), g->d_rowptr, rp.size() * 8, cudaMemcpyDeviceToHost));
  const int64_t* in_rp = rp.data();
  if (g->directed) {
    irp.resize(rp.size());
    LGBC_CUDA(cudaMemcpy(irp.data(), g->d_in_rowptr, irp.size() * 8, cudaMemcpyDeviceToHost));
    in_rp = irp.data();
  }
  return build_hubs(g, rp.data(), in_rp, g->tune.hub_degree);
}

HubData hub_data(const lgbc_graph* g) {
  HubData h;
  h.out_items = g->hubs.out_items;
  h.n_out = g->hubs.n_out;
  h.in_items = g->hubs.in_items;
  h.n_in = g->hubs.n_in;
  h.acc = g->hubs.acc;
  h.mask = g->hubs.mask;
  h.cnt = g->hubs.cnt;
  h.hub_degree = g->hubs.nslots > 0 ? g->hubs.built_for : INT32_MAX;
  h.dense_edges = g->tune.dense_edges;
  // low-degree graphs: segmented warps when the mean degree is below the cut
  h.segmented = g->n > 0 && g->nnz < static_cast<int64_t>(g->tune.segment_degree) * g->n ? 1 : 0;
  return h;
}

int read_ctl(lgbc_graph* g, const BatchCtl* dctl) {
  LGBC_CUDA(cudaMemcpyAsync(g->h_ctl, dctl, sizeof(BatchCtl), cudaMemcpyDeviceToHost, g->stream));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  return LGBC_OK;
}

int check_launch(lgbc_graph* g) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
  (void)g;
  return LGBC_OK;
}

MsBuffers ms_buffers(lgbc_graph* g, const int32_t* lane_src, const double* lane_w = nullptr) {
  MsWorkspace& w = g->ms;
  MsBuffers b;
  b.visit = w.visit;
  b.mb[0] = w.mb0;
  b.mb[1] = w.mb1;
  b.sigma = w.sigma;
  b.psi = w.psi;
  b.qv = w.qv;
  b.qm = w.qm;
  b.lvl_off = w.lvl_off;
  b.ctl = w.ctl;
  b.lane_src = lane_src;
  b.cap = w.cap;
  b.lane_w = lane_w;
  b.lane_w_n = 0;
  return b;
}

// Direction choice for the next level of a multi-source batch: bottom-up when
// the frontier's out-edges exceed the unfinished vertices' in-edges / alpha,
// back to top-down when the frontier is smaller than n / beta (Beamer,
// Asanovic & Patterson, SC 2012, applied to the union of the lanes).
bool choose_bottom_up(const lgbc_graph* g, const BatchCtl& c, bool was_bu) {
  const double mf = static_cast<double>(c.mf_cur);
  const double mu = static_cast<double>(g->nnz) - static_cast<double>(c.mu_done);
  const double nf = static_cast<double>(c.hi - c.lo);
  if (was_bu) return nf >= static_cast<double>(g->n) / g->tune.beta;
  return mf > mu / g->tune.alpha;
}

// One multi-source batch: forward level loop, then (with sigma) the backward
// dependency sweep into bc.  Returns LGBC_OK, or 1 when the batch must be
// replayed with FP64 path counts.
// Explicit (vertex, lane) seeds on the device, for unions of graphs.
struct Seeds {
  const int32_t* v = nullptr;
  const int32_t* lane = nullptr;
  int64_t count = 0;
  // optional premark of seedless lanes per component (unions of graphs)
  const int64_t* seg_off = nullptr;
  const uint64_t* seg_mark = nullptr;
  int64_t nseg = 0;
  // stacked unions with lane weights: one row of 64 weights per copy of an
  // lane_w_n-vertex graph, lane_w_count weights in all
  int64_t lane_w_n = 0;
  int64_t lane_w_count = 0;
};

// ---------------------------------------------------------------------------
// Device-driven level loops (tuning graph_loop = 1).  A forward sweep is one
// graph launch: WHILE(loop) { SWITCH(dir) { top-down level | bottom-up level };
// advance }, where the advance kernel also makes the direction choice and
// ends the loop when the sweep is done, a list must grow, a path count may
// overflow, or the level cap is reached.  A backward sweep is a second graph:
// WHILE(loop) { dependency level; level-- }, then the cleanup kernel.  The host
// reads the control block once per batch instead of once per level.
// ---------------------------------------------------------------------------
#define LOOP_CUDA(call)                                                              \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      if (graph) cudaGraphDestroy(graph);                                            \
      return cuda_fail(e_, #call);                                                   \
    }                                                                                \
  } while (0)

// Capture the kernels that `launch(stream)` queues into `into` after `deps`;
// returns the launch count of the capture.
template <class F>
int capture_into(lgbc_graph* g, cudaGraph_t into, const cudaGraphNode_t* deps, size_t ndeps,
                 F&& launch, int* count) {
  cudaError_t e = cudaStreamBeginCaptureToGraph(g->cap_stream, into, deps, nullptr, ndeps,
                                                cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCaptureToGraph");
  *count = launch(g->cap_stream);
  cudaGraph_t out = nullptr;
  e = cudaStreamEndCapture(g->cap_stream, &out);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  return LGBC_OK;
}

// The sink node of `graph` (its one node without dependents).
cudaGraphNode_t last_node(cudaGraph_t graph) {
  size_t count = 0;
  if (cudaGraphGetNodes(graph, nullptr, &count) != cudaSuccess || count == 0) return nullptr;
  std::vector<cudaGraphNode_t> nodes(count);
  if (cudaGraphGetNodes(graph, nodes.data(), &count) != cudaSuccess) return nullptr;
  // the nodes without dependents are the sinks; a chain has exactly one
  for (cudaGraphNode_t nd : nodes) {
    size_t nout = 0;
    if (cudaGraphNodeGetDependentNodes(nd, nullptr, nullptr, &nout) == cudaSuccess && nout == 0)
      return nd;
  }
  return nullptr;
}

int build_loop(lgbc_graph* g, const LoopKey& k, LoopGraph* out) {
  if (!g->cap_stream) {
    cudaError_t e = cudaStreamCreateWithFlags(&g->cap_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate (capture)");
  }
  cudaGraph_t graph = nullptr;
  LOOP_CUDA(cudaGraphCreate(&graph, 0));
  LoopParams lp{};
  // a handle belongs to the graph that holds its conditional node: `loop` to
  // the top-level graph, `dir` (forward) to the loop body
  LOOP_CUDA(cudaGraphConditionalHandleCreate(&lp.loop, graph, 0, cudaGraphCondAssignDefault));
  lp.n = g->n;
  lp.nnz = g->nnz;
  lp.alpha = k.alpha;
  lp.beta = k.beta;
  lp.sigma_kind = k.sigma_kind;
  lp.max_levels = g->n + 1;
  const DevGraph dg = g->dev();
  MsBuffers b = k.b;
  int cnt = 0;
  // arm
  int rc = capture_into(g, graph, nullptr, 0,
                        [&](cudaStream_t cs) {
                          return k.backward ? loop_back_arm(cs, b, lp) : loop_arm(cs, b, lp);
                        },
                        &cnt);
  if (rc != LGBC_OK) {
    cudaGraphDestroy(graph);
    return rc;
  }
  cudaGraphNode_t arm = last_node(graph);
  // WHILE node
  cudaGraphNodeParams wp{};
  wp.type = cudaGraphNodeTypeConditional;
  wp.conditional.handle = lp.loop;
  wp.conditional.type = cudaGraphCondTypeWhile;
  wp.conditional.size = 1;
  cudaGraphNode_t wnode = nullptr;
  LOOP_CUDA(cudaGraphAddNode(&wnode, graph, &arm, nullptr, 1, &wp));
  cudaGraph_t body = wp.conditional.phGraph_out[0];
  if (!k.backward) {
    LOOP_CUDA(cudaGraphConditionalHandleCreate(&lp.dir, body, 0, cudaGraphCondAssignDefault));
    cudaGraphNodeParams sp{};
    sp.type = cudaGraphNodeTypeConditional;
    sp.conditional.handle = lp.dir;
    sp.conditional.type = cudaGraphCondTypeSwitch;
    sp.conditional.size = 2;
    cudaGraphNode_t snode = nullptr;
    LOOP_CUDA(cudaGraphAddNode(&snode, body, nullptr, nullptr, 0, &sp));
    const HubData hd = k.hd;
    int32_t* dist = const_cast<int32_t*>(k.dist);
    rc = capture_into(g, sp.conditional.phGraph_out[0], nullptr, 0,
                      [&](cudaStream_t cs) {
                        return ms_topdown(g->cfg, cs, dg, b, hd, k.act, k.sigma_kind, dist, k.dist_ld);
                      },
                      &out->td_kernels);
    if (rc == LGBC_OK)
      rc = capture_into(g, sp.conditional.phGraph_out[1], nullptr, 0,
                        [&](cudaStream_t cs) {
                          return ms_bottomup(g->cfg, cs, dg, b, hd, k.act, k.sigma_kind, dist,
                                             k.dist_ld);
                        },
                        &out->bu_kernels);
    if (rc == LGBC_OK)
      rc = capture_into(g, body, &snode, 1,
                        [&](cudaStream_t cs) { return loop_advance(cs, b, lp); }, &cnt);
  } else {
    const HubData hd = k.hd;
    double* bc = const_cast<double*>(k.bc);
    rc = capture_into(g, body, nullptr, 0,
                      [&](cudaStream_t cs) {
                        return ms_backward_body(g->cfg, cs, dg, b, hd, k.sigma_kind, bc) +
                               loop_back_advance(cs, b, lp);
                      },
                      &out->body_kernels);
    if (rc == LGBC_OK)
      rc = capture_into(g, graph, &wnode, 1,
                        [&](cudaStream_t cs) { return ms_cleanup(g->cfg, cs, b); }, &cnt);
  }
  if (rc != LGBC_OK) {
    cudaGraphDestroy(graph);
    return rc;
  }
  cudaGraphExec_t exec = nullptr;
  LOOP_CUDA(cudaGraphInstantiate(&exec, graph, 0));
  out->key = k;
  out->graph = graph;
  out->exec = exec;
  return LGBC_OK;
}

// The cached loop for key k (built on first use; at most 8 are kept).
int get_loop(lgbc_graph* g, const LoopKey& k, LoopGraph** out) {
  for (auto& lg : g->loops)
    if (std::memcmp(&lg.key, &k, sizeof k) == 0) {
      lg.last_use = ++g->loop_clock;
      *out = &lg;
      return LGBC_OK;
    }
  if (g->loops.size() >= 8) {
    auto oldest = std::min_element(g->loops.begin(), g->loops.end(),
                                   [](const LoopGraph& a, const LoopGraph& b2) {
                                     return a.last_use < b2.last_use;
                                   });
    oldest->release();
    g->loops.erase(oldest);
  }
  LoopGraph lg;
  LGBC_TRY(build_loop(g, k, &lg));
  lg.last_use = ++g->loop_clock;
  g->loops.push_back(lg);
  *out = &g->loops.back();
  return LGBC_OK;
}

LoopKey loop_key(lgbc_graph* g, int backward, int sigma_kind, unsigned long long act,
                 const int32_t* dist, int64_t ld, const double* bc, const MsBuffers& b,
                 const HubData& hd) {
  LoopKey k;
  std::memset(&k, 0, sizeof k);  // padding bytes take part in the comparison
  k.backward = backward;
  k.sigma_kind = sigma_kind;
  k.act = act;
  k.dist = dist;
  k.dist_ld = ld;
  k.bc = bc;
  k.b = b;
  k.b.lane_src = nullptr;
  if (!backward) {  // the forward sweep never reads the weights
    k.b.lane_w = nullptr;
    k.b.lane_w_n = 0;
  }
  k.hd = hd;
  k.alpha = g->tune.alpha;
  k.beta = g->tune.beta;
  return k;
}

// lane_w (sigma batches): per-lane weights of the accumulation into bc.
// stats (distance-only batches): per-lane distance statistics, accumulated.
int run_ms_batch(lgbc_graph* g, const int32_t* lane_src, int nl, int sigma_kind, double* bc,
                 int32_t* dist, int64_t dist_ld, const Seeds& seeds = Seeds(),
                 const double* lane_w = nullptr, const LevelStats* stats = nullptr,
                 unsigned long long* stress = nullptr) {
  const DevGraph dg = g->dev();
  LGBC_TRY(ensure_hubs(g));
  const HubData hd = hub_data(g);
  const uint64_t act = nl >= 64 ? ~0ull : ((1ull << nl) - 1ull);
  for (;;) {
    MsBuffers b = ms_buffers(g, lane_src, lane_w);
    b.lane_w_n = seeds.lane_w_n;
    if (seeds.seg_mark) g->launches += ms_premark(g->cfg, g->stream, b, seeds.seg_off, seeds.seg_mark,
                                                  seeds.nseg);
    if (seeds.v)
      g->launches += ms_init_seeds(g->cfg, g->stream, dg, b, seeds.v, seeds.lane, seeds.count,
                                   sigma_kind, g->sigma_limit, dist, dist_ld);
    else
      g->launches += ms_init(g->stream, dg, b, nl, sigma_kind, g->sigma_limit, dist, dist_ld);
    LGBC_TRY(check_launch(g));
    // device-driven loops for plain batches (no weights, statistics or stress)
    if (g->tune.graph_loop == 1 && !stats && !stress) {
      MsBuffers bw = b;  // the backward graph reads the weights from a fixed buffer
      if (lane_w) {
        const int64_t cnt = seeds.lane_w_count > 0 ? seeds.lane_w_count : nl;
        if (cnt > g->d_lw_cap) {
          dev_free(g->d_lw_fixed);
          g->d_lw_cap = 0;
          LGBC_TRY(dev_alloc(&g->d_lw_fixed, static_cast<size_t>(std::max<int64_t>(cnt, 64))));
          g->d_lw_cap = std::max<int64_t>(cnt, 64);
        }
        LGBC_CUDA(cudaMemcpyAsync(g->d_lw_fixed, lane_w, static_cast<size_t>(cnt) * 8,
                                  cudaMemcpyDeviceToDevice, g->stream));
        bw.lane_w = g->d_lw_fixed;
      }
      LoopGraph* lg = nullptr;
      LGBC_TRY(get_loop(g, loop_key(g, 0, sigma_kind, act, dist, dist_ld, nullptr, b, hd), &lg));
      LGBC_CUDA(cudaGraphLaunch(lg->exec, g->stream));
      LGBC_TRY(check_launch(g));
      LGBC_TRY(read_ctl(g, b.ctl));
      const BatchCtl& c = *g->h_ctl;
      const int64_t lv = static_cast<int64_t>(c.td_levels + c.bu_levels);
      g->stats.levels += lv;
      g->stats.topdown_levels += static_cast<int64_t>(c.td_levels);
      g->stats.bottomup_levels += static_cast<int64_t>(c.bu_levels);
      g->launches += 1 + lv + static_cast<int64_t>(c.td_levels) * lg->td_kernels +
                     static_cast<int64_t>(c.bu_levels) * lg->bu_kernels;
      if (c.runaway) return fail(LGBC_ETIMEOUT, "forward sweep exceeded n + 1 levels");
      if (c.overflow_sigma && sigma_kind == kSigmaU64) {
        g->launches += ms_reset_all(g->stream, dg, b);
        return 1;
      }
      if (c.overflow_list) {
        LGBC_TRY(grow_ms_lists(g));
        g->launches += ms_reset_all(g->stream, dg, ms_buffers(g, lane_src));
        continue;
      }
      if (sigma_kind == kSigmaNone) {
        g->launches += ms_cleanup_all(g->cfg, g->stream, b);
        return check_launch(g);
      }
      const int maxl = c.maxlevel;
      LoopGraph* bg = nullptr;
      LGBC_TRY(get_loop(g, loop_key(g, 1, sigma_kind, act, nullptr, 0, bc, bw, hd), &bg));
      LGBC_CUDA(cudaGraphLaunch(bg->exec, g->stream));
      g->launches += 2 + static_cast<int64_t>(maxl + 1) * bg->body_kernels;
      if (seeds.seg_mark)  // premarked vertices were never listed: clear visit outright
        LGBC_CUDA(cudaMemsetAsync(b.visit, 0, static_cast<size_t>(g->n) * 8, g->stream));
      return check_launch(g);
    }
    bool bu = false;
    bool regrow = false;
    int64_t levels = 0;
    for (;;) {
      if (bu) {
        g->launches += ms_bottomup(g->cfg, g->stream, dg, b, hd, act, sigma_kind, dist, dist_ld);
        g->stats.bottomup_levels++;
      } else {
        g->launches += ms_topdown(g->cfg, g->stream, dg, b, hd, act, sigma_kind, dist, dist_ld);
        g->stats.topdown_levels++;
      }
      g->launches += ms_advance(g->stream, dg, b);
      LGBC_TRY(check_launch(g));
      LGBC_TRY(read_ctl(g, b.ctl));
      ++levels;
      // every level settles at least one new (vertex, lane) pair, so a sweep
      // longer than n + 1 levels can only mean a fault
      if (levels > g->n + 1) return fail(LGBC_ETIMEOUT, "forward sweep exceeded n + 1 levels");
      const BatchCtl& c = *g->h_ctl;
      if (c.overflow_sigma && sigma_kind == kSigmaU64) break;
      if (c.done) break;
      if (c.overflow_list) {
        regrow = true;
        break;
      }
      bu = choose_bottom_up(g, c, bu);
    }
    g->stats.levels += levels;
    if (regrow) {
      LGBC_TRY(grow_ms_lists(g));
      g->launches += ms_reset_all(g->stream, dg, ms_buffers(g, lane_src));
      continue;
    }
    if (g->h_ctl->overflow_sigma && sigma_kind == kSigmaU64) {
      g->launches += ms_reset_all(g->stream, dg, b);
      return 1;
    }
    if (sigma_kind == kSigmaNone && stress) {
      // stress sweep (distance-only forward, integer backward)
      const int maxl = g->h_ctl->maxlevel;
      g->launches += ms_begin_backward(g->stream, b);
      for (int L = maxl; L >= 0; --L)
        g->launches += st_backward_level(g->cfg, g->stream, dg, b, hd, stress);
      g->launches += ms_cleanup(g->cfg, g->stream, b);
      return check_launch(g);
    }
    if (sigma_kind == kSigmaNone) {
      if (stats) g->launches += ms_level_stats(g->cfg, g->stream, b, *stats);
      g->launches += ms_cleanup_all(g->cfg, g->stream, b);
      return check_launch(g);
    }
    const int maxl = g->h_ctl->maxlevel;
    g->launches += ms_begin_backward(g->stream, b);
    for (int L = maxl; L >= 0; --L)
      g->launches += ms_backward_level(g->cfg, g->stream, dg, b, hd, sigma_kind, bc);
    g->launches += ms_cleanup(g->cfg, g->stream, b);
    if (seeds.seg_mark)  // premarked vertices were never listed: clear visit outright
      LGBC_CUDA(cudaMemsetAsync(b.visit, 0, static_cast<size_t>(g->n) * 8, g->stream));
    return check_launch(g);
  }
}

// Brandes over the active sources already on the device (g->d_src[0, k)),
// accumulating into bc_dev (zeroed here); with d_w, source i's dependencies
// are scaled by d_w[i].
int run_stacked(lgbc_graph* g, int64_t copies, double* bc_dev, const std::vector<double>* w);

int run_betweenness(lgbc_graph* g, int64_t k_act, int endpoints, double* bc_dev,
                    const double* d_w = nullptr) {
  g->launches += fill_f64(g->cfg, g->stream, bc_dev, g->n, 0.0);
  const int lanes0 = std::max(1, std::min<int>(kMaxLanes, g->tune.lanes));
  const int64_t batches = (k_act + lanes0 - 1) / lanes0;
  const int64_t copies = g->n > 0 ? std::min<int64_t>(g->tune.stack_vertices / g->n, batches) : 0;
  const bool host_w = d_w && static_cast<int64_t>(g->h_weights.size()) == k_act;
  if ((!d_w || host_w) && copies >= 4 && static_cast<int64_t>(g->h_active.size()) == k_act) {
    LGBC_TRY(run_stacked(g, copies, bc_dev, d_w ? &g->h_weights : nullptr));
    if (endpoints) g->launches += add_endpoints(g->cfg, g->stream, bc_dev, g->n, g->d_src, k_act);
    return check_launch(g);
  }
  if (k_act > 0) LGBC_TRY(ensure_ms(g, true));
  const int lanes = std::max(1, std::min<int>(kMaxLanes, g->tune.lanes));
  for (int64_t s0 = 0; s0 < k_act; s0 += lanes) {
    const int nl = static_cast<int>(std::min<int64_t>(lanes, k_act - s0));
    const double* lw = d_w ? d_w + s0 : nullptr;
    int rc = run_ms_batch(g, g->d_src + s0, nl, kSigmaU64, bc_dev, nullptr, 0, Seeds(), lw);
    if (rc == 1) {
      g->stats.wide_batches++;
      rc = run_ms_batch(g, g->d_src + s0, nl, kSigmaF64, bc_dev, nullptr, 0, Seeds(), lw);
    }
    if (rc != LGBC_OK) return rc;
    g->stats.batches++;
  }
  if (endpoints) g->launches += add_endpoints(g->cfg, g->stream, bc_dev, g->n, g->d_src, k_act);
  return check_launch(g);
}

// BFS distances from the landmarks (computed once per graph, kept on the device).
int ensure_landmarks(lgbc_graph* g) {
  if (g->d_lmdist || g->landmarks.empty()) return LGBC_OK;
  const int nl = static_cast<int>(g->landmarks.size());
  LGBC_TRY(ensure_ms(g, false));
  int32_t* d_lm = nullptr;
  LGBC_TRY(dev_alloc(&d_lm, static_cast<size_t>(nl)));
  std::unique_ptr<int32_t, void (*)(int32_t*)> guard(d_lm, [](int32_t* q) { cudaFree(q); });
  LGBC_CUDA(cudaMemcpyAsync(d_lm, g->landmarks.data(), static_cast<size_t>(nl) * 4,
                            cudaMemcpyHostToDevice, g->stream));
  int32_t* d = nullptr;
  LGBC_TRY(dev_alloc(&d, static_cast<size_t>(nl) * static_cast<size_t>(g->n)));
  g->launches += fill_i32(g->cfg, g->stream, d, static_cast<int64_t>(nl) * g->n, kUnreached);
  const lgbc_stats saved = g->stats;  // the call's statistics describe its own sources
  const int rc = run_ms_batch(g, d_lm, nl, kSigmaNone, nullptr, d, g->n);
  g->stats = saved;
  if (rc != LGBC_OK) {
    cudaFree(d);
    return rc;
  }
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  g->d_lmdist = d;
  return LGBC_OK;
}

// Source ordering (tuning source_order = 1): sort the active sources by
// their distance vectors to the landmarks (lexicographically, then by id),
// so that a 64-lane batch holds sources with similar distance profiles.  Such
// sources reach a vertex at fewer distinct levels, and every distinct level
// costs the vertex one pass over its edges in each sweep.  `w`, when given,
// is permuted alongside.
int order_active(lgbc_graph* g, std::vector<int32_t>& act, std::vector<double>* w) {
  const int64_t k = static_cast<int64_t>(act.size());
  if (g->tune.source_order == 0 || k <= g->tune.lanes || g->landmarks.empty()) return LGBC_OK;
  LGBC_TRY(ensure_landmarks(g));
  const int nl = static_cast<int>(g->landmarks.size());
  int32_t* d_buf = nullptr;  // k sources | k x nl keys
  LGBC_TRY(dev_alloc(&d_buf, static_cast<size_t>(k) * static_cast<size_t>(nl + 1)));
  std::unique_ptr<int32_t, void (*)(int32_t*)> guard(d_buf, [](int32_t* q) { cudaFree(q); });
  LGBC_CUDA(cudaMemcpyAsync(d_buf, act.data(), static_cast<size_t>(k) * 4, cudaMemcpyHostToDevice,
                            g->stream));
  g->launches += gather_cols(g->cfg, g->stream, g->d_lmdist, g->n, nl, d_buf, k, d_buf + k);
  std::vector<int32_t> key(static_cast<size_t>(k) * static_cast<size_t>(nl));
  LGBC_CUDA(cudaMemcpyAsync(key.data(), d_buf + k, key.size() * 4, cudaMemcpyDeviceToHost,
                            g->stream));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  std::vector<int64_t> perm(static_cast<size_t>(k));
  for (int64_t i = 0; i < k; ++i) perm[static_cast<size_t>(i)] = i;
  std::stable_sort(perm.begin(), perm.end(), [&](int64_t a, int64_t b) {
    const int32_t* ka = key.data() + a * nl;
    const int32_t* kb = key.data() + b * nl;
    for (int j = 0; j < nl; ++j)
      if (ka[j] != kb[j]) return ka[j] < kb[j];
    return act[static_cast<size_t>(a)] < act[static_cast<size_t>(b)];
  });
  std::vector<int32_t> a2(static_cast<size_t>(k));
  for (int64_t i = 0; i < k; ++i) a2[static_cast<size_t>(i)] = act[static_cast<size_t>(perm[i])];
  act.swap(a2);
  if (w) {
    std::vector<double> w2(static_cast<size_t>(k));
    for (int64_t i = 0; i < k; ++i) w2[static_cast<size_t>(i)] = (*w)[static_cast<size_t>(perm[i])];
    w->swap(w2);
  }
  return LGBC_OK;
}

// Stacked batches for small graphs: the active sources (g->h_active, in
// their batch order) run as a disjoint union of `copies` copies of the graph;
// in union batch u, copy r holds the sources of ordinary batch u * copies + r
// (one lane each, as in lgbc_betweenness_many), lanes without a source in a
// copy are premarked there, and the copies' raw vectors are summed at the end.
// Each union batch does the work of `copies` batches with the launches of one.
int run_stacked(lgbc_graph* g, int64_t copies, double* bc_dev, const std::vector<double>* w) {
  const int64_t n = g->n, nnz = g->nnz;
  const int L = std::max(1, std::min<int>(kMaxLanes, g->tune.lanes));
  if (!g->stack || g->stack_copies != copies) {
    if (g->stack) lgbc_graph_destroy(g->stack);
    g->stack = nullptr;
    g->stack_copies = 0;
    // replicate the CSR(s) on the host: copy r holds vertices [r n, (r + 1) n)
    std::vector<int64_t> rp(static_cast<size_t>(n + 1)), irp;
    std::vector<int32_t> ci(static_cast<size_t>(nnz)), ici;
    LGBC_CUDA(cudaMemcpy(rp.data(), g->d_rowptr, rp.size() * 8, cudaMemcpyDeviceToHost));
    if (nnz) LGBC_CUDA(cudaMemcpy(ci.data(), g->d_colidx, ci.size() * 4, cudaMemcpyDeviceToHost));
    if (g->directed) {
      irp.resize(rp.size());
      ici.resize(ci.size());
      LGBC_CUDA(cudaMemcpy(irp.data(), g->d_in_rowptr, irp.size() * 8, cudaMemcpyDeviceToHost));
      if (nnz)
        LGBC_CUDA(cudaMemcpy(ici.data(), g->d_in_colidx, ici.size() * 4, cudaMemcpyDeviceToHost));
    }
    auto replicate = [&](const std::vector<int64_t>& r0, const std::vector<int32_t>& c0,
                         std::vector<int64_t>& r1, std::vector<int32_t>& c1) {
      r1.resize(static_cast<size_t>(copies * n + 1));
      c1.resize(static_cast<size_t>(copies * nnz));
      for (int64_t r = 0; r < copies; ++r) {
        for (int64_t v = 0; v < n; ++v) r1[static_cast<size_t>(r * n + v)] = r * nnz + r0[static_cast<size_t>(v)];
        for (int64_t e = 0; e < nnz; ++e)
          c1[static_cast<size_t>(r * nnz + e)] = static_cast<int32_t>(r * n + c0[static_cast<size_t>(e)]);
      }
      r1[static_cast<size_t>(copies * n)] = copies * nnz;
    };
    std::vector<int64_t> srp, sirp;
    std::vector<int32_t> sci, sici;
    replicate(rp, ci, srp, sci);
    if (g->directed) replicate(irp, ici, sirp, sici);
    lgbc_graph* st = nullptr;
    LGBC_TRY(lgbc_graph_create(&st, copies * n, copies * nnz, srp.data(), sci.data(),
                               g->directed ? sirp.data() : nullptr,
                               g->directed ? sici.data() : nullptr, g->directed));
    g->stack = st;
    g->stack_copies = copies;
  }
  lgbc_graph* st = g->stack;
  st->tune = g->tune;
  st->tune.source_order = 0;
  st->tune.stack_vertices = 0;
  LGBC_CUDA(cudaSetDevice(g->device));
  // seeds and premarks of every union batch
  const std::vector<int32_t>& act = g->h_active;
  const int64_t k = static_cast<int64_t>(act.size());
  const int64_t per = L * copies;
  const int64_t nbu = (k + per - 1) / per;
  std::vector<int32_t> sv, sl;
  std::vector<int64_t> bstart(static_cast<size_t>(nbu + 1), 0), voff(static_cast<size_t>(copies + 1));
  std::vector<uint64_t> marks(static_cast<size_t>(nbu * copies));
  std::vector<int64_t> filled(static_cast<size_t>(nbu), 0);  // ordinary batches per union batch
  // lane weights: row u * copies + r holds copy r's 64 lanes of union batch u
  std::vector<double> wrows(w ? static_cast<size_t>(nbu * copies * 64) : 0, 0.0);
  for (int64_t r = 0; r <= copies; ++r) voff[static_cast<size_t>(r)] = r * n;
  for (int64_t u = 0; u < nbu; ++u) {
    for (int64_t r = 0; r < copies; ++r) {
      if ((u * copies + r) * L < k) filled[static_cast<size_t>(u)]++;
      uint64_t seeded = 0;
      const int64_t i0 = (u * copies + r) * L;
      for (int l = 0; l < L && i0 + l < k; ++l) {
        sv.push_back(static_cast<int32_t>(r * n + act[static_cast<size_t>(i0 + l)]));
        sl.push_back(l);
        seeded |= 1ull << l;
        if (w) wrows[static_cast<size_t>((u * copies + r) * 64 + l)] = (*w)[static_cast<size_t>(i0 + l)];
      }
      const uint64_t all = L >= 64 ? ~0ull : ((1ull << L) - 1ull);
      marks[static_cast<size_t>(u * copies + r)] = all & ~seeded;
    }
    bstart[static_cast<size_t>(u + 1)] = static_cast<int64_t>(sv.size());
  }
  // one device buffer: weight rows | voff | marks | seed vertices | seed lanes
  const size_t bytes = wrows.size() * 8 + voff.size() * 8 + marks.size() * 8 + sv.size() * 4 +
                       sl.size() * 4 + 16;
  unsigned char* buf = nullptr;
  LGBC_TRY(dev_alloc(&buf, bytes));
  std::unique_ptr<unsigned char, cudaError_t (*)(void*)> guard(buf, cudaFree);
  double* d_wrows = reinterpret_cast<double*>(buf);
  if (!wrows.empty())
    LGBC_CUDA(cudaMemcpyAsync(d_wrows, wrows.data(), wrows.size() * 8, cudaMemcpyHostToDevice,
                              st->stream));
  int64_t* d_voff = reinterpret_cast<int64_t*>(buf + wrows.size() * 8);
  uint64_t* d_marks = reinterpret_cast<uint64_t*>(d_voff + voff.size());
  int32_t* d_sv = reinterpret_cast<int32_t*>(d_marks + marks.size());
  int32_t* d_sl = d_sv + sv.size();
  LGBC_CUDA(cudaMemcpyAsync(d_voff, voff.data(), voff.size() * 8, cudaMemcpyHostToDevice, st->stream));
  LGBC_CUDA(cudaMemcpyAsync(d_marks, marks.data(), marks.size() * 8, cudaMemcpyHostToDevice, st->stream));
  LGBC_CUDA(cudaMemcpyAsync(d_sv, sv.data(), sv.size() * 4, cudaMemcpyHostToDevice, st->stream));
  LGBC_CUDA(cudaMemcpyAsync(d_sl, sl.data(), sl.size() * 4, cudaMemcpyHostToDevice, st->stream));
  if (!st->d_bc) LGBC_TRY(dev_alloc(&st->d_bc, static_cast<size_t>(st->n)));
  st->launches += fill_f64(st->cfg, st->stream, st->d_bc, st->n, 0.0);
  LGBC_TRY(ensure_ms(st, true));
  // the caller's stream waits for nothing of ours: order the two streams
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  for (int64_t u = 0; u < nbu; ++u) {
    Seeds sd;
    sd.v = d_sv + bstart[static_cast<size_t>(u)];
    sd.lane = d_sl + bstart[static_cast<size_t>(u)];
    sd.count = bstart[static_cast<size_t>(u + 1)] - bstart[static_cast<size_t>(u)];
    sd.seg_off = d_voff;
    sd.seg_mark = d_marks + static_cast<size_t>(u * copies);
    sd.nseg = copies;
    const double* lw = nullptr;
    if (w) {
      lw = d_wrows + u * copies * 64;
      sd.lane_w_n = n;
      sd.lane_w_count = copies * 64;
    }
    int rc = run_ms_batch(st, nullptr, L, kSigmaU64, st->d_bc, nullptr, 0, sd, lw);
    if (rc == 1) {
      g->stats.wide_batches++;
      rc = run_ms_batch(st, nullptr, L, kSigmaF64, st->d_bc, nullptr, 0, sd, lw);
    }
    if (rc != LGBC_OK) {
      g->launches += st->launches;
      st->launches = 0;
      return rc;
    }
    g->stats.batches += filled[static_cast<size_t>(u)];  // counted as ordinary batches
  }
  LGBC_CUDA(cudaStreamSynchronize(st->stream));
  g->stats.levels += st->stats.levels;
  g->stats.topdown_levels += st->stats.topdown_levels;
  g->stats.bottomup_levels += st->stats.bottomup_levels;
  st->stats = lgbc_stats{};
  g->launches += st->launches + 1;
  st->launches = 0;
  sum_copies(g->cfg, g->stream, st->d_bc, n, copies, bc_dev);
  return check_launch(g);
}

// Host-side part shared by the betweenness entry points: validate, filter
// degree-0 sources (betweenness.jl:58), order and upload the active list.
int prepare_sources(lgbc_graph* g, const int32_t* src, int64_t nsrc, int64_t* k_act) {
  std::vector<int32_t> active;
  if (!src) {
    active.reserve(static_cast<size_t>(g->n));
    for (int64_t v = 0; v < g->n; ++v)
      if (g->has_degree[static_cast<size_t>(v)]) active.push_back(static_cast<int32_t>(v));
  } else {
    LGBC_TRY(check_sources(g, src, nsrc));
    active.reserve(static_cast<size_t>(nsrc));
    for (int64_t i = 0; i < nsrc; ++i)
      if (g->has_degree[static_cast<size_t>(src[i])]) active.push_back(src[i]);
  }
  LGBC_TRY(order_active(g, active, nullptr));
  *k_act = static_cast<int64_t>(active.size());
  g->h_active = active;
  g->h_weights.clear();
  LGBC_TRY(ensure_src(g, *k_act));
  if (*k_act > 0)
    LGBC_CUDA(cudaMemcpyAsync(g->d_src, active.data(), active.size() * sizeof(int32_t),
                              cudaMemcpyHostToDevice, g->stream));
  // the pageable source vector must outlive the copy
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  return LGBC_OK;
}

void reset_stats(lgbc_graph* g) {
  g->stats = lgbc_stats{};
  g->stats.kernel_launches = g->launches;
}

void finish_stats(lgbc_graph* g) { g->stats.kernel_launches = g->launches - g->stats.kernel_launches; }

// Fills a freshly constructed handle; on failure the caller destroys it.
// Device, stream, events and launch shape of a new handle.
int init_handle(lgbc_graph* g, int64_t n, int directed) {
  LGBC_CUDA(cudaGetDevice(&g->device));
  g->n = n;
  g->directed = directed ? 1 : 0;
  cudaDeviceProp prop;
  LGBC_CUDA(cudaGetDeviceProperties(&prop, g->device));
  g->cfg.sms = prop.multiProcessorCount;
  g->cfg.block = 256;
  g->cfg.grid = prop.multiProcessorCount * 8;
  g->max_smem = prop.sharedMemPerBlockOptin;
  bfs_configure(g->max_smem);
  LGBC_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
  LGBC_CUDA(cudaEventCreate(&g->ev_start));
  LGBC_CUDA(cudaEventCreate(&g->ev_stop));
  LGBC_CUDA(cudaMallocHost(reinterpret_cast<void**>(&g->h_ctl), sizeof(BatchCtl)));
  return LGBC_OK;
}

// Host-side bookkeeping from the row pointers: degree filter, path-count
// bound, landmarks and the hub table.
int finish_handle(lgbc_graph* g, const int64_t* rowptr, const int64_t* in_rowptr);

int create_impl(lgbc_graph* g, int64_t n, int64_t nnz, const int64_t* rowptr, const int32_t* colidx,
                const int64_t* in_rowptr, const int32_t* in_colidx, int directed) {
  LGBC_TRY(init_handle(g, n, directed));
  g->nnz = nnz;

  LGBC_TRY(dev_alloc(&g->d_rowptr, static_cast<size_t>(n + 1)));
  LGBC_TRY(dev_alloc(&g->d_colidx, static_cast<size_t>(nnz)));
  LGBC_CUDA(cudaMemcpyAsync(g->d_rowptr, rowptr, static_cast<size_t>(n + 1) * 8,
                            cudaMemcpyHostToDevice, g->stream));
  if (nnz > 0)
    LGBC_CUDA(cudaMemcpyAsync(g->d_colidx, colidx, static_cast<size_t>(nnz) * 4,
                              cudaMemcpyHostToDevice, g->stream));
  if (directed) {
    LGBC_TRY(dev_alloc(&g->d_in_rowptr, static_cast<size_t>(n + 1)));
    LGBC_TRY(dev_alloc(&g->d_in_colidx, static_cast<size_t>(nnz)));
    LGBC_CUDA(cudaMemcpyAsync(g->d_in_rowptr, in_rowptr, static_cast<size_t>(n + 1) * 8,
                              cudaMemcpyHostToDevice, g->stream));
    if (nnz > 0)
      LGBC_CUDA(cudaMemcpyAsync(g->d_in_colidx, in_colidx, static_cast<size_t>(nnz) * 4,
                                cudaMemcpyHostToDevice, g->stream));
  } else {
    g->d_in_rowptr = g->d_rowptr;
    g->d_in_colidx = g->d_colidx;
  }
  // the CSR is validated on the device: one pass over rowptr / colidx
  int* d_bad = nullptr;
  LGBC_TRY(dev_alloc(&d_bad, 1));
  cudaMemsetAsync(d_bad, 0, sizeof(int), g->stream);
  g->launches += validate_csr(g->cfg, g->stream, g->d_rowptr, g->d_colidx, n, nnz, d_bad);
  if (directed)
    g->launches += validate_csr(g->cfg, g->stream, g->d_in_rowptr, g->d_in_colidx, n, nnz, d_bad);
  int bad = 0;
  cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, g->stream);
  cudaError_t e = cudaStreamSynchronize(g->stream);
  cudaFree(d_bad);
  if (e != cudaSuccess) return cuda_fail(e, "graph upload");
  LGBC_TRY(check_launch(g));
  if (bad & 1) return fail(LGBC_EINVAL, "rowptr must be non-decreasing");
  if (bad & 2) return fail(LGBC_EINVAL, "column index out of range");
  return finish_handle(g, rowptr, directed ? in_rowptr : rowptr);
}

int finish_handle(lgbc_graph* g, const int64_t* rowptr, const int64_t* in_rowptr) {
  const int64_t n = g->n;
  const int directed = g->directed;
  // degree(g, v) > 0: in+out for digraphs (src/core.jl:66-67), kept on the host
  g->has_degree.assign(static_cast<size_t>(n), 0);
  int64_t max_in = 0;
  for (int64_t v = 0; v < n; ++v) {
    const int64_t dout = rowptr[v + 1] - rowptr[v];
    const int64_t din = directed ? in_rowptr[v + 1] - in_rowptr[v] : dout;
    const int64_t d = directed ? dout + din : dout;
    g->has_degree[static_cast<size_t>(v)] = d > 0 ? 1 : 0;
    max_in = std::max(max_in, din);
  }
  g->sigma_limit = ~0ull / static_cast<unsigned long long>(max_in + 1);
  {
    // the kLandmarks highest-degree vertices (ties: smaller id), for source ordering
    std::vector<std::pair<int64_t, int32_t>> top;
    for (int64_t v = 0; v < n; ++v) {
      const int64_t d = (rowptr[v + 1] - rowptr[v]) + (directed ? in_rowptr[v + 1] - in_rowptr[v] : 0);
      if (d == 0) continue;
      const std::pair<int64_t, int32_t> item(-d, static_cast<int32_t>(v));
      if (top.size() < static_cast<size_t>(kLandmarks)) {
        top.push_back(item);
        std::push_heap(top.begin(), top.end());
      } else if (item < top.front()) {
        std::pop_heap(top.begin(), top.end());
        top.back() = item;
        std::push_heap(top.begin(), top.end());
      }
    }
    std::sort(top.begin(), top.end());
    for (const auto& t : top) g->landmarks.push_back(t.second);
  }
  return build_hubs(g, rowptr, directed ? in_rowptr : rowptr, g->tune.hub_degree);
}

}  // namespace

extern "C" {

const char* lgbc_version(void) { return "lgbc 0.1.0 sm_103a"; }

const char* lgbc_last_error(void) { return g_last_error.c_str(); }

int lgbc_device_count(void) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return count;
}

int lgbc_graph_create(lgbc_graph** out, int64_t n, int64_t nnz, const int64_t* rowptr,
                      const int32_t* colidx, const int64_t* in_rowptr, const int32_t* in_colidx,
                      int directed) {
  if (!out) return fail(LGBC_EINVAL, "null output handle pointer");
  *out = nullptr;
  if (n < 0 || nnz < 0) return fail(LGBC_EINVAL, "negative vertex or edge count");
  if (n >= INT32_MAX) return fail(LGBC_EINVAL, "vertex ids must fit in int32");
  if (!rowptr || (nnz > 0 && !colidx)) return fail(LGBC_EINVAL, "null CSR array");
  if (directed && (!in_rowptr || (nnz > 0 && !in_colidx)))
    return fail(LGBC_EINVAL, "a directed graph needs its in-CSR (badjlist)");
  if (rowptr[0] != 0 || rowptr[n] != nnz) return fail(LGBC_EINVAL, "rowptr must run from 0 to nnz");
  if (directed && (in_rowptr[0] != 0 || in_rowptr[n] != nnz))
    return fail(LGBC_EINVAL, "in_rowptr must run from 0 to nnz");

  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(LGBC_ECUDA, std::string("no CUDA device available: ") +
                                (e != cudaSuccess ? cudaGetErrorString(e) : "0 devices"));
  }
  lgbc_graph* g = new (std::nothrow) lgbc_graph();
  if (!g) return fail(LGBC_ENOMEM, "host allocation failed");
  const int rc = create_impl(g, n, nnz, rowptr, colidx, in_rowptr, in_colidx, directed);
  if (rc != LGBC_OK) {
    const std::string msg = g_last_error;
    lgbc_graph_destroy(g);
    g_last_error = msg;
    return rc;
  }
  *out = g;
  return LGBC_OK;
}

int lgbc_graph_destroy(lgbc_graph* g) {
  if (!g) return LGBC_OK;
  cudaSetDevice(g->device);
  if (g->stream) cudaStreamSynchronize(g->stream);
  g->ms.release();
  g->bfs.release();
  g->hubs.release();
  g->learned.release();
  for (auto& lg : g->loops) lg.release();
  g->loops.clear();
  if (g->stack) lgbc_graph_destroy(g->stack);
  g->stack = nullptr;
  if (g->cap_stream) cudaStreamDestroy(g->cap_stream);
  if (g->d_in_rowptr != g->d_rowptr) dev_free(g->d_in_rowptr);
  if (g->d_in_colidx != g->d_colidx) dev_free(g->d_in_colidx);
  dev_free(g->d_rowptr);
  dev_free(g->d_colidx);
  dev_free(g->d_src);
  dev_free(g->d_bc);
  dev_free(g->d_dist);
  dev_free(g->d_lmdist);
  dev_free(g->d_lw_fixed);
  if (g->h_ctl) cudaFreeHost(g->h_ctl);
  if (g->ev_start) cudaEventDestroy(g->ev_start);
  if (g->ev_stop) cudaEventDestroy(g->ev_stop);
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
  return LGBC_OK;
}

int lgbc_graph_info(const lgbc_graph* g, int64_t* n, int64_t* nnz, int* directed) {
  LGBC_TRY(check_graph(g));
  if (n) *n = g->n;
  if (nnz) *nnz = g->nnz;
  if (directed) *directed = g->directed;
  return LGBC_OK;
}

}  // extern "C"

namespace {

// Level-synchronous BFS over dg from d_src[0, nsrc) into d_dist, which the
// caller has filled (kUnreached, and any other value on vertices the search
// must treat as already visited).
int run_bfs(lgbc_graph* g, const DevGraph& dg, int64_t nsrc) {
  BfsBuffers b{g->bfs.queue, {g->bfs.bm0, g->bfs.bm1}, g->bfs.ctl};
  g->launches += bfs_init(g->cfg, g->stream, dg, b, g->d_src, nsrc, g->d_dist);
  LGBC_TRY(check_launch(g));
  LGBC_TRY(read_ctl(g, b.ctl));
  const size_t bm_bytes = static_cast<size_t>(((g->n + 31) / 32 + 3) & ~int64_t(3)) * 4;
  const int stage = bm_bytes <= g->max_smem ? 1 : 0;
  bool bu = false;
  while (!g->h_ctl->done) {
    const BatchCtl& c = *g->h_ctl;
    const double mf = static_cast<double>(c.mf_cur);
    const double mu = static_cast<double>(g->nnz) - static_cast<double>(c.mu_done);
    const double nf = static_cast<double>(c.hi - c.lo);
    bu = bu ? (nf >= static_cast<double>(g->n) / g->tune.beta) : (mf > mu / g->tune.alpha);
    if (bu) {
      g->launches += bfs_bottomup(g->cfg, g->stream, dg, b, g->d_dist, stage);
      g->stats.bottomup_levels++;
    } else {
      g->launches += bfs_topdown(g->cfg, g->stream, dg, b, g->d_dist);
      g->stats.topdown_levels++;
    }
    g->launches += bfs_advance(g->stream, b);
    LGBC_TRY(check_launch(g));
    LGBC_TRY(read_ctl(g, b.ctl));
    g->stats.levels++;
    if (g->stats.levels > g->n + 1) return fail(LGBC_ETIMEOUT, "BFS exceeded n + 1 levels");
  }
  return LGBC_OK;
}

// Upload nsrc sources and fill the distance buffer with kUnreached.
int prepare_bfs(lgbc_graph* g, const int32_t* src, int64_t nsrc) {
  LGBC_TRY(ensure_bfs(g));
  LGBC_TRY(ensure_dist(g, g->n));
  LGBC_TRY(ensure_src(g, nsrc));
  if (nsrc > 0)
    LGBC_CUDA(cudaMemcpyAsync(g->d_src, src, static_cast<size_t>(nsrc) * 4, cudaMemcpyHostToDevice,
                              g->stream));
  g->launches += fill_i32(g->cfg, g->stream, g->d_dist, g->n, kUnreached);
  return LGBC_OK;
}

}  // namespace

extern "C" {

int lgbc_gdistances(lgbc_graph* g, const int32_t* src, int64_t nsrc, int32_t* dist_out) {
  LGBC_TRY(check_graph(g));
  std::lock_guard<std::mutex> lock(g->mu);
  LGBC_TRY(use_device(g));
  if (!dist_out && g->n > 0) return fail(LGBC_EINVAL, "null output");
  LGBC_TRY(check_sources(g, src, nsrc));
  reset_stats(g);
  if (g->n == 0) return LGBC_OK;
  LGBC_TRY(prepare_bfs(g, src, nsrc));
  LGBC_TRY(run_bfs(g, g->dev(), nsrc));
  LGBC_CUDA(cudaMemcpyAsync(dist_out, g->d_dist, static_cast<size_t>(g->n) * 4,
                            cudaMemcpyDeviceToHost, g->stream));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  finish_stats(g);
  return LGBC_OK;
}

int lgbc_gdistances_batch(lgbc_graph* g, const int32_t* src, int64_t nsrc, int32_t* dist_out) {
  LGBC_TRY(check_graph(g));
  std::lock_guard<std::mutex> lock(g->mu);
  LGBC_TRY(use_device(g));
  LGBC_TRY(check_sources(g, src, nsrc));
  if (nsrc > 0 && g->n > 0 && !dist_out) return fail(LGBC_EINVAL, "null output");
  reset_stats(g);
  if (nsrc == 0 || g->n == 0) return LGBC_OK;
  LGBC_TRY(ensure_ms(g, false));
  LGBC_TRY(ensure_src(g, nsrc));
  LGBC_CUDA(cudaMemcpyAsync(g->d_src, src, static_cast<size_t>(nsrc) * 4, cudaMemcpyHostToDevice,
                            g->stream));
  const int lanes = kMaxLanes;
  LGBC_TRY(ensure_dist(g, static_cast<int64_t>(lanes) * g->n));
  for (int64_t s0 = 0; s0 < nsrc; s0 += lanes) {
    const int nl = static_cast<int>(std::min<int64_t>(lanes, nsrc - s0));
    g->launches += fill_i32(g->cfg, g->stream, g->d_dist, static_cast<int64_t>(nl) * g->n, kUnreached);
    LGBC_TRY(run_ms_batch(g, g->d_src + s0, nl, kSigmaNone, nullptr, g->d_dist, g->n));
    LGBC_CUDA(cudaMemcpyAsync(dist_out + s0 * g->n, g->d_dist,
                              static_cast<size_t>(nl) * static_cast<size_t>(g->n) * 4,
                              cudaMemcpyDeviceToHost, g->stream));
    g->stats.batches++;
  }
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  finish_stats(g);
  return LGBC_OK;
}

int lgbc_betweenness_dev(lgbc_graph* g, const int32_t* src, int64_t nsrc, int endpoints,
                         double* bc_raw_dev) {
  LGBC_TRY(check_graph(g));
  std::lock_guard<std::mutex> lock(g->mu);
  LGBC_TRY(use_device(g));
  if (!bc_raw_dev && g->n > 0) return fail(LGBC_EINVAL, "null output");
  reset_stats(g);
  int64_t k_act = 0;
  LGBC_TRY(prepare_sources(g, src, nsrc, &k_act));
  g->stats.active_sources = k_act;
  LGBC_TRY(run_betweenness(g, k_act, endpoints, bc_raw_dev));
  finish_stats(g);
  return LGBC_OK;
}

int lgbc_betweenness(lgbc_graph* g, const int32_t* src, int64_t nsrc, int endpoints,
                     double* bc_raw_out) {
  LGBC_TRY(check_graph(g));
  std::lock_guard<std::mutex> lock(g->mu);
  LGBC_TRY(use_device(g));
  if (!bc_raw_out && g->n > 0) return fail(LGBC_EINVAL, "null output");
  reset_stats(g);
  int64_t k_act = 0;
  LGBC_TRY(prepare_sources(g, src, nsrc, &k_act));
  g->stats.active_sources = k_act;
  if (g->n == 0) return LGBC_OK;
  if (!g->d_bc) LGBC_TRY(dev_alloc(&g->d_bc, static_cast<size_t>(g->n)));
  LGBC_TRY(run_betweenness(g, k_act, endpoints, g->d_bc));
  LGBC_CUDA(cudaMemcpyAsync(bc_raw_out, g->d_bc, static_cast<size_t>(g->n) * 8,
                            cudaMemcpyDeviceToHost, g->stream));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  finish_stats(g);
  return LGBC_OK;
}

int lgbc_graph_sync(lgbc_graph* g) {
  LGBC_TRY(check_graph(g));
  LGBC_TRY(use_device(g));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  return LGBC_OK;
}

int lgbc_timer_start(lgbc_graph* g) {
  LGBC_TRY(check_graph(g));
  LGBC_TRY(use_device(g));
  g->launches_at_start = g->launches;
  LGBC_CUDA(cudaEventRecord(g->ev_start, g->stream));
  return LGBC_OK;
}

int lgbc_timer_stop(lgbc_graph* g, double* elapsed_ms, int64_t* kernel_launches) {
  LGBC_TRY(check_graph(g));
  LGBC_TRY(use_device(g));
  LGBC_CUDA(cudaEventRecord(g->ev_stop, g->stream));
  LGBC_CUDA(cudaEventSynchronize(g->ev_stop));
  float ms = 0.f;
  LGBC_CUDA(cudaEventElapsedTime(&ms, g->ev_start, g->ev_stop));
  if (elapsed_ms) *elapsed_ms = ms;
  if (kernel_launches) *kernel_launches = g->launches - g->launches_at_start;
  return LGBC_OK;
}

int lgbc_graph_stats(const lgbc_graph* g, lgbc_stats* out) {
  LGBC_TRY(check_graph(g));
  if (!out) return fail(LGBC_EINVAL, "null output");
  *out = g->stats;
  return LGBC_OK;
}

int lgbc_get_tuning(const lgbc_graph* g, lgbc_tuning* out) {
  LGBC_TRY(check_graph(g));
  if (!out) return fail(LGBC_EINVAL, "null output");
  *out = g->tune;
  return LGBC_OK;
}

int lgbc_set_tuning(lgbc_graph* g, const lgbc_tuning* t) {
  LGBC_TRY(check_graph(g));
  if (!t) return fail(LGBC_EINVAL, "null tuning");
  if (!(t->alpha > 0) || !(t->beta > 0) || t->lanes < 1 || t->lanes > kMaxLanes ||
      t->hub_degree < 1 || t->dense_edges < 0 || t->segment_degree < 0 ||
      (t->source_order != 0 && t->source_order != 1) || (t->graph_loop != 0 && t->graph_loop != 1) ||
      t->stack_vertices < 0)
    return fail(LGBC_EINVAL,
                "tuning out of range (alpha, beta > 0; 1 <= lanes <= 64; hub_degree >= 1; dense_edges >= 0)");
  std::lock_guard<std::mutex> lock(g->mu);
  g->tune = *t;
  return LGBC_OK;
}

int lgbc_device_alloc(void** ptr, int64_t bytes) {
  if (!ptr || bytes < 0) return fail(LGBC_EINVAL, "bad allocation request");
  cudaError_t e = cudaMalloc(ptr, static_cast<size_t>(std::max<int64_t>(bytes, 1)));
  if (e != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return fail(LGBC_ENOMEM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
  }
  return LGBC_OK;
}

int lgbc_device_free(void* ptr) {
  if (ptr) LGBC_CUDA(cudaFree(ptr));
  return LGBC_OK;
}

int lgbc_host_alloc(void** ptr, int64_t bytes) {
  if (!ptr || bytes < 0) return fail(LGBC_EINVAL, "bad allocation request");
  cudaError_t e = cudaMallocHost(ptr, static_cast<size_t>(std::max<int64_t>(bytes, 1)));
  if (e != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return fail(LGBC_ENOMEM, std::string("cudaMallocHost failed: ") + cudaGetErrorString(e));
  }
  return LGBC_OK;
}

int lgbc_host_free(void* ptr) {
  if (ptr) LGBC_CUDA(cudaFreeHost(ptr));
  return LGBC_OK;
}

int lgbc_memcpy(void* dst, const void* src, int64_t bytes, int kind) {
  if (bytes < 0 || (bytes > 0 && (!dst || !src))) return fail(LGBC_EINVAL, "bad copy request");
  cudaMemcpyKind k;
  switch (kind) {
    case 1: k = cudaMemcpyHostToDevice; break;
    case 2: k = cudaMemcpyDeviceToHost; break;
    case 3: k = cudaMemcpyDeviceToDevice; break;
    default: return fail(LGBC_EINVAL, "copy kind must be 1, 2 or 3");
  }
  if (bytes > 0) LGBC_CUDA(cudaMemcpy(dst, src, static_cast<size_t>(bytes), k));
  return LGBC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Exact betweenness of many graphs (disjoint unions, one lane per source
// index in every graph of a group).
// ---------------------------------------------------------------------------
namespace {

struct ManyGraph {
  int64_t idx, n, nnz;
  const int64_t* rowptr;  // n + 1 entries, local
  const int32_t* colidx;  // local ids
  int64_t out_off;        // position of its first vertex in bc_raw_out
};

// Source ordering inside a union of graphs: graph k's active sources are
// sorted by their BFS distances to graph k's own kLandmarks highest-degree
// vertices (one seeded kLandmarks-lane distance batch serves every graph of
// the union at once), so that a batch lane pairs sources with similar
// distance profiles in every component, as order_active does for one graph.
int order_many(lgbc_graph* g, const std::vector<ManyGraph>& grp, const std::vector<int64_t>& voff,
               std::vector<std::vector<int32_t>>& act) {
  const int nl = kLandmarks;
  std::vector<int32_t> sv, sl;
  for (size_t k = 0; k < grp.size(); ++k) {
    std::vector<std::pair<int64_t, int32_t>> deg;
    for (int64_t v = 0; v < grp[k].n; ++v) {
      const int64_t d = grp[k].rowptr[v + 1] - grp[k].rowptr[v];
      if (d > 0) deg.emplace_back(-d, static_cast<int32_t>(v));
    }
    const size_t top = std::min<size_t>(deg.size(), static_cast<size_t>(nl));
    std::partial_sort(deg.begin(), deg.begin() + static_cast<std::ptrdiff_t>(top), deg.end());
    for (size_t j = 0; j < top; ++j) {
      sv.push_back(static_cast<int32_t>(voff[k] + deg[j].second));
      sl.push_back(static_cast<int32_t>(j));
    }
  }
  if (sv.empty()) return LGBC_OK;
  const int64_t N = g->n;
  LGBC_TRY(ensure_ms(g, false));
  int32_t* d_dist = nullptr;  // nl x N distances | seeds | lanes
  LGBC_TRY(dev_alloc(&d_dist, static_cast<size_t>(nl) * static_cast<size_t>(N) + 2 * sv.size()));
  std::unique_ptr<int32_t, cudaError_t (*)(void*)> guard(d_dist, cudaFree);
  int32_t* d_sv = d_dist + static_cast<int64_t>(nl) * N;
  int32_t* d_sl = d_sv + sv.size();
  LGBC_CUDA(cudaMemcpyAsync(d_sv, sv.data(), sv.size() * 4, cudaMemcpyHostToDevice, g->stream));
  LGBC_CUDA(cudaMemcpyAsync(d_sl, sl.data(), sl.size() * 4, cudaMemcpyHostToDevice, g->stream));
  g->launches += fill_i32(g->cfg, g->stream, d_dist, static_cast<int64_t>(nl) * N, kUnreached);
  Seeds sd;
  sd.v = d_sv;
  sd.lane = d_sl;
  sd.count = static_cast<int64_t>(sv.size());
  LGBC_TRY(run_ms_batch(g, nullptr, nl, kSigmaNone, nullptr, d_dist, N, sd));
  std::vector<int32_t> dist(static_cast<size_t>(nl) * static_cast<size_t>(N));
  LGBC_CUDA(cudaMemcpyAsync(dist.data(), d_dist, dist.size() * 4, cudaMemcpyDeviceToHost, g->stream));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  for (size_t k = 0; k < grp.size(); ++k) {
    auto& a = act[k];
    const int64_t base = voff[k];
    std::stable_sort(a.begin(), a.end(), [&](int32_t x, int32_t y) {
      for (int j = 0; j < nl; ++j) {
        const int32_t dx = dist[static_cast<size_t>(j) * N + base + x];
        const int32_t dy = dist[static_cast<size_t>(j) * N + base + y];
        if (dx != dy) return dx < dy;
      }
      return x < y;
    });
  }
  return LGBC_OK;
}

int many_group(const std::vector<ManyGraph>& grp, int endpoints, double* bc_raw_out) {
  // union CSR on the host
  int64_t N = 0, NNZ = 0;
  for (const auto& m : grp) {
    N += m.n;
    NNZ += m.nnz;
  }
  std::vector<int64_t> rp(static_cast<size_t>(N + 1));
  std::vector<int32_t> ci(static_cast<size_t>(NNZ));
  std::vector<int64_t> voff(grp.size() + 1);
  int64_t vo = 0, eo = 0;
  for (size_t k = 0; k < grp.size(); ++k) {
    const ManyGraph& m = grp[k];
    voff[k] = vo;
    for (int64_t v = 0; v < m.n; ++v) rp[static_cast<size_t>(vo + v)] = eo + m.rowptr[v];
    for (int64_t e = 0; e < m.nnz; ++e) {
      // a local id outside [0, n) would land in a neighbouring graph of the union
      if (m.colidx[e] < 0 || m.colidx[e] >= m.n)
        return fail(LGBC_EINVAL, "graph " + std::to_string(m.idx) + ": column index outside [0, n)");
      ci[static_cast<size_t>(eo + e)] = static_cast<int32_t>(vo + m.colidx[e]);
    }
    vo += m.n;
    eo += m.nnz;
  }
  voff[grp.size()] = vo;
  rp[static_cast<size_t>(N)] = NNZ;
  lgbc_graph* g = nullptr;
  LGBC_TRY(lgbc_graph_create(&g, N, NNZ, rp.data(), ci.data(), nullptr, nullptr, 0));
  std::unique_ptr<lgbc_graph, int (*)(lgbc_graph*)> guard(g, lgbc_graph_destroy);
  std::lock_guard<std::mutex> lock(g->mu);

  // every graph's active sources (degree > 0), and the endpoint terms
  std::vector<std::vector<int32_t>> act(grp.size());
  std::vector<int32_t> sv, sl, act_src;
  std::vector<double> seg_add(grp.size()), src_add;
  int64_t maxa = 0;
  for (size_t k = 0; k < grp.size(); ++k) {
    for (int64_t v = 0; v < grp[k].n; ++v)
      if (g->has_degree[static_cast<size_t>(voff[k] + v)]) {
        act[k].push_back(static_cast<int32_t>(v));
        act_src.push_back(static_cast<int32_t>(voff[k] + v));
        src_add.push_back(static_cast<double>(grp[k].n) - 2.0);
      }
    seg_add[k] = static_cast<double>(act[k].size());
    maxa = std::max<int64_t>(maxa, static_cast<int64_t>(act[k].size()));
  }
  if (g->tune.source_order == 1 && maxa > kMaxLanes)
    LGBC_TRY(order_many(g, grp, voff, act));
  // batch b, lane l holds the (64 b + l)-th ordered source of every graph
  const int64_t nb = (maxa + kMaxLanes - 1) / kMaxLanes;
  std::vector<int64_t> bstart(static_cast<size_t>(nb + 1), 0);
  std::vector<uint64_t> marks(static_cast<size_t>(nb) * grp.size());
  for (int64_t b = 0; b < nb; ++b) {
    for (size_t k = 0; k < grp.size(); ++k) {
      uint64_t seeded = 0;
      for (int l = 0; l < kMaxLanes; ++l) {
        const int64_t i = b * kMaxLanes + l;
        if (i < static_cast<int64_t>(act[k].size())) {
          sv.push_back(static_cast<int32_t>(voff[k] + act[k][static_cast<size_t>(i)]));
          sl.push_back(l);
          seeded |= 1ull << l;
        }
      }
      marks[static_cast<size_t>(b) * grp.size() + k] = ~seeded;
    }
    bstart[static_cast<size_t>(b + 1)] = static_cast<int64_t>(sv.size());
  }
  int64_t* d_voff = nullptr;
  uint64_t* d_marks = nullptr;
  LGBC_TRY(dev_alloc(&d_voff, voff.size()));
  std::unique_ptr<int64_t, cudaError_t (*)(void*)> g7(d_voff, cudaFree);
  LGBC_TRY(dev_alloc(&d_marks, marks.size()));
  std::unique_ptr<uint64_t, cudaError_t (*)(void*)> g8(d_marks, cudaFree);
  LGBC_CUDA(cudaMemcpyAsync(d_voff, voff.data(), voff.size() * 8, cudaMemcpyHostToDevice, g->stream));
  if (!marks.empty())
    LGBC_CUDA(cudaMemcpyAsync(d_marks, marks.data(), marks.size() * 8, cudaMemcpyHostToDevice,
                              g->stream));
  int32_t* d_sv = nullptr;
  int32_t* d_sl = nullptr;
  LGBC_TRY(dev_alloc(&d_sv, sv.size()));
  std::unique_ptr<int32_t, cudaError_t (*)(void*)> g1(d_sv, cudaFree);
  LGBC_TRY(dev_alloc(&d_sl, sl.size()));
  std::unique_ptr<int32_t, cudaError_t (*)(void*)> g2(d_sl, cudaFree);
  if (!sv.empty()) {
    LGBC_CUDA(cudaMemcpyAsync(d_sv, sv.data(), sv.size() * 4, cudaMemcpyHostToDevice, g->stream));
    LGBC_CUDA(cudaMemcpyAsync(d_sl, sl.data(), sl.size() * 4, cudaMemcpyHostToDevice, g->stream));
  }
  if (!g->d_bc) LGBC_TRY(dev_alloc(&g->d_bc, static_cast<size_t>(N)));
  g->launches += fill_f64(g->cfg, g->stream, g->d_bc, N, 0.0);
  if (!sv.empty()) LGBC_TRY(ensure_ms(g, true));
  for (int64_t b = 0; b < nb; ++b) {
    Seeds sd;
    sd.v = d_sv + bstart[static_cast<size_t>(b)];
    sd.lane = d_sl + bstart[static_cast<size_t>(b)];
    sd.count = bstart[static_cast<size_t>(b + 1)] - bstart[static_cast<size_t>(b)];
    if (sd.count == 0) continue;
    sd.seg_off = d_voff;
    sd.seg_mark = d_marks + static_cast<size_t>(b) * grp.size();
    sd.nseg = static_cast<int64_t>(grp.size());
    int rc = run_ms_batch(g, nullptr, kMaxLanes, kSigmaU64, g->d_bc, nullptr, 0, sd);
    if (rc == 1) rc = run_ms_batch(g, nullptr, kMaxLanes, kSigmaF64, g->d_bc, nullptr, 0, sd);
    if (rc != LGBC_OK) return rc;
  }
  if (endpoints && !act_src.empty()) {
    int64_t* d_off = nullptr;
    double* d_add = nullptr;
    int32_t* d_src = nullptr;
    double* d_sadd = nullptr;
    LGBC_TRY(dev_alloc(&d_off, voff.size()));
    std::unique_ptr<int64_t, cudaError_t (*)(void*)> g3(d_off, cudaFree);
    LGBC_TRY(dev_alloc(&d_add, seg_add.size()));
    std::unique_ptr<double, cudaError_t (*)(void*)> g4(d_add, cudaFree);
    LGBC_TRY(dev_alloc(&d_src, act_src.size()));
    std::unique_ptr<int32_t, cudaError_t (*)(void*)> g5(d_src, cudaFree);
    LGBC_TRY(dev_alloc(&d_sadd, src_add.size()));
    std::unique_ptr<double, cudaError_t (*)(void*)> g6(d_sadd, cudaFree);
    LGBC_CUDA(cudaMemcpyAsync(d_off, voff.data(), voff.size() * 8, cudaMemcpyHostToDevice, g->stream));
    LGBC_CUDA(cudaMemcpyAsync(d_add, seg_add.data(), seg_add.size() * 8, cudaMemcpyHostToDevice, g->stream));
    LGBC_CUDA(cudaMemcpyAsync(d_src, act_src.data(), act_src.size() * 4, cudaMemcpyHostToDevice, g->stream));
    LGBC_CUDA(cudaMemcpyAsync(d_sadd, src_add.data(), src_add.size() * 8, cudaMemcpyHostToDevice, g->stream));
    g->launches += add_endpoints_many(g->cfg, g->stream, g->d_bc, d_off, d_add,
                                      static_cast<int64_t>(grp.size()), d_src, d_sadd,
                                      static_cast<int64_t>(act_src.size()));
    LGBC_CUDA(cudaStreamSynchronize(g->stream));
  }
  std::vector<double> out(static_cast<size_t>(N));
  LGBC_CUDA(cudaMemcpyAsync(out.data(), g->d_bc, static_cast<size_t>(N) * 8, cudaMemcpyDeviceToHost,
                            g->stream));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  for (size_t k = 0; k < grp.size(); ++k)
    std::memcpy(bc_raw_out + grp[k].out_off, out.data() + voff[k],
                static_cast<size_t>(grp[k].n) * 8);
  return LGBC_OK;
}

}  // namespace

extern "C" int lgbc_betweenness_many(int64_t ngraphs, const int64_t* n, const int64_t* rowptr_off,
                                     const int64_t* col_off, const int64_t* rowptr,
                                     const int32_t* colidx, int endpoints, double* bc_raw_out) {
  if (ngraphs < 0) return fail(LGBC_EINVAL, "negative graph count");
  if (ngraphs == 0) return LGBC_OK;
  if (!n || !rowptr_off || !col_off || !rowptr || !bc_raw_out)
    return fail(LGBC_EINVAL, "null argument");
  std::vector<ManyGraph> gs(static_cast<size_t>(ngraphs));
  int64_t out = 0;
  for (int64_t i = 0; i < ngraphs; ++i) {
    if (n[i] < 0 || rowptr_off[i] < 0 || col_off[i] < 0) return fail(LGBC_EINVAL, "negative offset");
    const int64_t* rp = rowptr + rowptr_off[i];
    if (rp[0] != 0) return fail(LGBC_EINVAL, "each graph's rowptr must start at 0");
    gs[static_cast<size_t>(i)] =
        ManyGraph{i, n[i], rp[n[i]], rp, colidx ? colidx + col_off[i] : nullptr, out};
    if (gs[static_cast<size_t>(i)].nnz > 0 && !colidx) return fail(LGBC_EINVAL, "null colidx");
    out += n[i];
  }
  // size-sorted groups of at most kGroupVertices vertices (one big graph alone)
  std::vector<size_t> order(gs.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t a, size_t b) { return gs[a].n > gs[b].n; });
  const int64_t kGroupVertices = int64_t(1) << 21;
  std::vector<ManyGraph> grp;
  int64_t gv = 0;
  for (size_t oi = 0; oi < order.size(); ++oi) {
    const ManyGraph& m = gs[order[oi]];
    if (!grp.empty() && gv + m.n > kGroupVertices) {
      LGBC_TRY(many_group(grp, endpoints, bc_raw_out));
      grp.clear();
      gv = 0;
    }
    grp.push_back(m);
    gv += m.n;
  }
  if (!grp.empty()) LGBC_TRY(many_group(grp, endpoints, bc_raw_out));
  return LGBC_OK;
}

// ---------------------------------------------------------------------------
// Learned source proposal (learned.cu, mlp.cu)
// ---------------------------------------------------------------------------
namespace {

int ensure_learned(lgbc_graph* g) {
  LearnedWorkspace& w = g->learned;
  if (w.core) return LGBC_OK;
  const size_t n = static_cast<size_t>(g->n);
  const size_t tiles = static_cast<size_t>(proposal_tiles(g->n));
  LGBC_TRY(dev_alloc(&w.core, n));
  LGBC_TRY(dev_alloc(&w.flag, n));
  LGBC_TRY(dev_alloc(&w.list, n));
  LGBC_TRY(dev_alloc(&w.counters, 4));
  LGBC_TRY(dev_alloc(&w.feat, n));
  LGBC_TRY(dev_alloc(&w.y, n));
  LGBC_TRY(dev_alloc(&w.fscr, tiles + 1));
  LGBC_TRY(dev_alloc(&w.e, n));
  LGBC_TRY(dev_alloc(&w.tsum, tiles));
  LGBC_TRY(dev_alloc(&w.scal, 1));
  LGBC_TRY(dev_alloc(&w.p, n));
  LGBC_TRY(dev_alloc(&w.cdf, n));
  LGBC_CUDA(cudaMemsetAsync(w.flag, 0, n, g->stream));
  return LGBC_OK;
}

unsigned long long read_counter(lgbc_graph* g, int i, int* rc) {
  unsigned long long v = 0;
  cudaError_t e = cudaMemcpyAsync(&v, g->learned.counters + i, 8, cudaMemcpyDeviceToHost, g->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
  *rc = e == cudaSuccess ? LGBC_OK : cuda_fail(e, "reading a device counter");
  return v;
}

// Core numbers into learned.core: degrees without self-loops, then h-index
// passes over the flagged vertices until none is lowered.  strict: a
// self-loop is an error (core_number's ArgumentError).
int compute_core(lgbc_graph* g, bool strict) {
  LearnedWorkspace& w = g->learned;
  const DevGraph dg = g->dev();
  LGBC_CUDA(cudaMemsetAsync(w.counters, 0, 4 * 8, g->stream));
  g->launches += core_degree(g->cfg, g->stream, dg, w.core, reinterpret_cast<int*>(w.counters));
  LGBC_TRY(check_launch(g));
  int rc = LGBC_OK;
  const unsigned long long loops = read_counter(g, 0, &rc);
  LGBC_TRY(rc);
  if (strict && (loops & 0xffffffffull))
    return fail(LGBC_EINVAL, "core_number: graph must not have self-loops");
  const int32_t* list = nullptr;
  int64_t nlist = g->n;
  w.core_passes = 0;
  while (nlist > 0) {
    g->launches += core_pass(g->cfg, g->stream, dg, list, nlist, w.core, w.flag, w.counters + 1);
    LGBC_CUDA(cudaMemsetAsync(w.counters + 2, 0, 8, g->stream));
    g->launches += core_compact(g->cfg, g->stream, g->n, w.flag, w.list, w.counters + 2);
    LGBC_TRY(check_launch(g));
    nlist = static_cast<int64_t>(read_counter(g, 2, &rc));
    LGBC_TRY(rc);
    list = w.list;
    // every pass with work lowers some value by at least one; the values
    // start at the degrees, so more passes than stored entries means a fault
    if (++w.core_passes > g->nnz + 2) return fail(LGBC_ETIMEOUT, "core iteration did not settle");
  }
  return LGBC_OK;
}

int compute_features(lgbc_graph* g) {
  LGBC_TRY(ensure_learned(g));
  LGBC_TRY(compute_core(g, false));
  g->launches += features(g->cfg, g->stream, g->dev(), g->learned.core, g->learned.feat);
  return check_launch(g);
}

// Per-source distance statistics over the multi-source BFS (no path counts):
// vertices reached at levels >= 1, the sum and the maximum of their levels.
int distance_stats(lgbc_graph* g, const int32_t* src, int64_t nsrc,
                   std::vector<unsigned long long>* cnt, std::vector<unsigned long long>* dsum,
                   std::vector<int>* dmax) {
  cnt->assign(static_cast<size_t>(nsrc), 0ull);
  dsum->assign(static_cast<size_t>(nsrc), 0ull);
  dmax->assign(static_cast<size_t>(nsrc), 0);
  if (nsrc == 0) return LGBC_OK;
  LGBC_TRY(ensure_ms(g, false));
  LGBC_TRY(ensure_src(g, nsrc));
  unsigned long long* buf = nullptr;  // cnt | dsum | dmax (as int)
  LGBC_TRY(dev_alloc(&buf, static_cast<size_t>(nsrc) * 3));
  std::unique_ptr<unsigned long long, void (*)(unsigned long long*)> guard(
      buf, [](unsigned long long* q) { cudaFree(q); });
  LGBC_CUDA(cudaMemsetAsync(buf, 0, static_cast<size_t>(nsrc) * 24, g->stream));
  LGBC_CUDA(cudaMemcpyAsync(g->d_src, src, static_cast<size_t>(nsrc) * 4, cudaMemcpyHostToDevice,
                            g->stream));
  int* dm = reinterpret_cast<int*>(buf + 2 * nsrc);
  for (int64_t s0 = 0; s0 < nsrc; s0 += kMaxLanes) {
    const int nl = static_cast<int>(std::min<int64_t>(kMaxLanes, nsrc - s0));
    const LevelStats st{buf + s0, buf + nsrc + s0, dm + s0};
    LGBC_TRY(run_ms_batch(g, g->d_src + s0, nl, kSigmaNone, nullptr, nullptr, 0, Seeds(), nullptr,
                          &st));
    g->stats.batches++;
  }
  LGBC_CUDA(cudaMemcpyAsync(cnt->data(), buf, static_cast<size_t>(nsrc) * 8, cudaMemcpyDeviceToHost,
                            g->stream));
  LGBC_CUDA(cudaMemcpyAsync(dsum->data(), buf + nsrc, static_cast<size_t>(nsrc) * 8,
                            cudaMemcpyDeviceToHost, g->stream));
  LGBC_CUDA(cudaMemcpyAsync(dmax->data(), dm, static_cast<size_t>(nsrc) * 4, cudaMemcpyDeviceToHost,
                            g->stream));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  return LGBC_OK;
}

int need_undirected(const lgbc_graph* g, const char* what) {
  if (g->directed) return fail(LGBC_EINVAL, std::string(what) + " covers undirected graphs");
  return LGBC_OK;
}

}  // namespace

extern "C" {

int lgbc_core_number(lgbc_graph* g, int32_t* core_out) {
  LGBC_TRY(check_graph(g));
  std::lock_guard<std::mutex> lock(g->mu);
  LGBC_TRY(use_device(g));
  if (!core_out && g->n > 0) return fail(LGBC_EINVAL, "null output");
  reset_stats(g);
  if (g->n == 0) return LGBC_OK;
  LGBC_TRY(ensure_learned(g));
  LGBC_TRY(compute_core(g, true));
  LGBC_CUDA(cudaMemcpyAsync(core_out, g->learned.core, static_cast<size_t>(g->n) * 4,
                            cudaMemcpyDeviceToHost, g->stream));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  g->stats.levels = g->learned.core_passes;
  finish_stats(g);
  return LGBC_OK;
}

int lgbc_features(lgbc_graph* g, float* feat_out) {
  LGBC_TRY(check_graph(g));
  std::lock_guard<std::mutex> lock(g->mu);
  LGBC_TRY(use_device(g));
  LGBC_TRY(need_undirected(g, "lgbc_features"));
  if (!feat_out && g->n > 0) return fail(LGBC_EINVAL, "null output");
  reset_stats(g);
  if (g->n == 0) return LGBC_OK;
  LGBC_TRY(compute_features(g));
  LGBC_CUDA(cudaMemcpyAsync(feat_out, g->learned.feat, static_cast<size_t>(g->n) * 16,
                            cudaMemcpyDeviceToHost, g->stream));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  g->stats.levels = g->learned.core_passes;
  finish_stats(g);
  return LGBC_OK;
}

int lgbc_distance_stats(lgbc_graph* g, const int32_t* src, int64_t nsrc, int64_t* reached_out,
                        int64_t* dsum_out, int32_t* dmax_out) {
  LGBC_TRY(check_graph(g));
  std::lock_guard<std::mutex> lock(g->mu);
  LGBC_TRY(use_device(g));
  LGBC_TRY(check_sources(g, src, nsrc));
  reset_stats(g);
  std::vector<unsigned long long> cnt, dsum;
  std::vector<int> dmax;
  LGBC_TRY(distance_stats(g, src, nsrc, &cnt, &dsum, &dmax));
  for (int64_t i = 0; i < nsrc; ++i) {
    const size_t k = static_cast<size_t>(i);
    if (reached_out) reached_out[i] = static_cast<int64_t>(cnt[k]) + 1;
    if (dsum_out) dsum_out[i] = static_cast<int64_t>(dsum[k]);
    if (dmax_out) dmax_out[i] = dmax[k];
  }
  finish_stats(g);
  return LGBC_OK;
}

int lgbc_dependency_mass(lgbc_graph* g, const int32_t* src, int64_t nsrc, double* mass_out) {
  LGBC_TRY(check_graph(g));
  std::lock_guard<std::mutex> lock(g->mu);
  LGBC_TRY(use_device(g));
  LGBC_TRY(check_sources(g, src, nsrc));
  if (nsrc > 0 && !mass_out) return fail(LGBC_EINVAL, "null output");
  reset_stats(g);
  std::vector<unsigned long long> cnt, dsum;
  std::vector<int> dmax;
  LGBC_TRY(distance_stats(g, src, nsrc, &cnt, &dsum, &dmax));
  // sum over reached t != s of (d - 1)
  for (int64_t i = 0; i < nsrc; ++i)
    mass_out[i] = static_cast<double>(dsum[static_cast<size_t>(i)] - cnt[static_cast<size_t>(i)]);
  finish_stats(g);
  return LGBC_OK;
}

int lgbc_betweenness_weighted(lgbc_graph* g, const int32_t* src, const double* w, int64_t nsrc,
                              double* bc_raw_out) {
  LGBC_TRY(check_graph(g));
  std::lock_guard<std::mutex> lock(g->mu);
  LGBC_TRY(use_device(g));
  if (!bc_raw_out && g->n > 0) return fail(LGBC_EINVAL, "null output");
  LGBC_TRY(check_sources(g, src, nsrc));
  if (nsrc > 0 && !w) return fail(LGBC_EINVAL, "null weights");
  for (int64_t i = 0; i < nsrc; ++i)
    if (!std::isfinite(w[i])) return fail(LGBC_EINVAL, "non-finite weight");
  reset_stats(g);
  if (g->n == 0) return LGBC_OK;
  // degree-0 sources contribute nothing (betweenness.jl:58): drop them with
  // their weights.  Repeats of a source are merged into one lane carrying the
  // summed weight (sum_i w_i delta_{s_i} is unchanged; a sample drawn with
  // replacement repeats its likeliest sources).
  std::vector<std::pair<int32_t, double>> sw;
  sw.reserve(static_cast<size_t>(nsrc));
  for (int64_t i = 0; i < nsrc; ++i)
    if (g->has_degree[static_cast<size_t>(src[i])]) sw.emplace_back(src[i], w[i]);
  std::stable_sort(sw.begin(), sw.end(),
                   [](const std::pair<int32_t, double>& a, const std::pair<int32_t, double>& b) {
                     return a.first < b.first;
                   });
  std::vector<int32_t> act;
  std::vector<double> aw;
  act.reserve(sw.size());
  aw.reserve(sw.size());
  for (const auto& e : sw) {
    if (!act.empty() && act.back() == e.first) {
      aw.back() += e.second;
    } else {
      act.push_back(e.first);
      aw.push_back(e.second);
    }
  }
  LGBC_TRY(order_active(g, act, &aw));
  const int64_t k_act = static_cast<int64_t>(act.size());
  g->stats.active_sources = k_act;
  g->h_active = act;
  g->h_weights = aw;
  LGBC_TRY(ensure_src(g, k_act));
  double* d_w = nullptr;
  LGBC_TRY(dev_alloc(&d_w, static_cast<size_t>(std::max<int64_t>(k_act, 1))));
  std::unique_ptr<double, void (*)(double*)> guard(d_w, [](double* q) { cudaFree(q); });
  if (k_act > 0) {
    LGBC_CUDA(cudaMemcpyAsync(g->d_src, act.data(), static_cast<size_t>(k_act) * 4,
                              cudaMemcpyHostToDevice, g->stream));
    LGBC_CUDA(cudaMemcpyAsync(d_w, aw.data(), static_cast<size_t>(k_act) * 8, cudaMemcpyHostToDevice,
                              g->stream));
  }
  if (!g->d_bc) LGBC_TRY(dev_alloc(&g->d_bc, static_cast<size_t>(g->n)));
  LGBC_TRY(run_betweenness(g, k_act, 0, g->d_bc, d_w));
  LGBC_CUDA(cudaMemcpyAsync(bc_raw_out, g->d_bc, static_cast<size_t>(g->n) * 8,
                            cudaMemcpyDeviceToHost, g->stream));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  finish_stats(g);
  return LGBC_OK;
}

int lgbc_proposal_build(lgbc_graph* g, lgbc_mlp* m, double eps, double* p_out) {
  LGBC_TRY(check_graph(g));
  std::lock_guard<std::mutex> lock(g->mu);
  LGBC_TRY(use_device(g));
  LGBC_TRY(need_undirected(g, "the learned proposal"));
  if (!(eps >= 0.0 && eps <= 1.0)) return fail(LGBC_EINVAL, "eps must be in [0, 1]");
  MlpView mv;
  LGBC_TRY(mlp_view(m, &mv));
  if (mv.device != g->device) return fail(LGBC_EINVAL, "MLP and graph live on different devices");
  reset_stats(g);
  if (g->n == 0) return fail(LGBC_EINVAL, "empty graph");
  g->learned.built = false;
  LGBC_TRY(compute_features(g));
  LearnedWorkspace& w = g->learned;
  g->launches += mlp_forward(g->cfg, g->stream, w.feat, g->n, mv.P, mv.norm, w.y);
  g->launches += proposal_build(g->stream, w.y, g->n, eps, w.fscr, w.e, w.tsum, w.scal, w.p, w.cdf);
  LGBC_TRY(check_launch(g));
  if (p_out)
    LGBC_CUDA(cudaMemcpyAsync(p_out, w.p, static_cast<size_t>(g->n) * 8, cudaMemcpyDeviceToHost,
                              g->stream));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  w.built = true;
  g->stats.levels = w.core_passes;
  finish_stats(g);
  return LGBC_OK;
}

int lgbc_proposal_sample(lgbc_graph* g, int64_t k, uint64_t seed, int scheme, int32_t* src_out,
                         double* w_out) {
  LGBC_TRY(check_graph(g));
  std::lock_guard<std::mutex> lock(g->mu);
  LGBC_TRY(use_device(g));
  LearnedWorkspace& w = g->learned;
  if (!w.built) return fail(LGBC_EINVAL, "no proposal built for this graph");
  if (k < 0 || (k > 0 && (!src_out || !w_out))) return fail(LGBC_EINVAL, "bad sample count or null output");
  if (scheme != LGBC_SAMPLE_IID && scheme != LGBC_SAMPLE_SYSTEMATIC)
    return fail(LGBC_EINVAL, "unknown sampling scheme");
  reset_stats(g);
  if (k == 0) return LGBC_OK;
  if (k > w.samp_cap) {
    dev_free(w.samp);
    dev_free(w.samp_w);
    w.samp_cap = 0;
    LGBC_TRY(dev_alloc(&w.samp, static_cast<size_t>(k)));
    LGBC_TRY(dev_alloc(&w.samp_w, static_cast<size_t>(k)));
    w.samp_cap = k;
  }
  g->launches += proposal_sample(g->stream, w.cdf, w.p, g->n, k, seed,
                                 scheme == LGBC_SAMPLE_SYSTEMATIC, w.samp, w.samp_w);
  LGBC_TRY(check_launch(g));
  LGBC_CUDA(cudaMemcpyAsync(src_out, w.samp, static_cast<size_t>(k) * 4, cudaMemcpyDeviceToHost,
                            g->stream));
  LGBC_CUDA(cudaMemcpyAsync(w_out, w.samp_w, static_cast<size_t>(k) * 8, cudaMemcpyDeviceToHost,
                            g->stream));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  finish_stats(g);
  return LGBC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Autotuner
// ---------------------------------------------------------------------------
namespace {

// Identifies a graph shape and device for the tuning cache.
std::string tune_signature(const lgbc_graph* g) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, g->device) != cudaSuccess) prop.multiProcessorCount = 0;
  char buf[256];
  std::snprintf(buf, sizeof buf, "n=%lld,nnz=%lld,dir=%d,sms=%d", static_cast<long long>(g->n),
                static_cast<long long>(g->nnz), g->directed, prop.multiProcessorCount);
  return buf;
}

bool tune_from_cache(const char* path, const std::string& sig, lgbc_tuning* out) {
  if (!path) return false;
  FILE* f = std::fopen(path, "r");
  if (!f) return false;
  char line[512];
  bool found = false;
  while (std::fgets(line, sizeof line, f)) {
    char key[256];
    lgbc_tuning t{};
    if (std::sscanf(line, "%255s %lf %lf %d %d %d %d %d %d %d", key, &t.alpha, &t.beta,
                    &t.hub_degree, &t.lanes, &t.dense_edges, &t.segment_degree, &t.source_order,
                    &t.graph_loop, &t.stack_vertices) == 10 &&
        sig == key && t.alpha > 0 && t.beta > 0 && t.lanes >= 1 && t.lanes <= kMaxLanes &&
        t.hub_degree >= 1 && t.dense_edges >= 0 && t.segment_degree >= 0 &&
        (t.source_order == 0 || t.source_order == 1) && (t.graph_loop == 0 || t.graph_loop == 1) &&
        t.stack_vertices >= 0) {
      *out = t;  // the last matching line wins
      found = true;
    }
  }
  std::fclose(f);
  return found;
}

// Milliseconds of one Brandes pass over the k sources already in d_src with
// tuning t (best of `reps`, after one unmeasured pass).
int tune_measure(lgbc_graph* g, const lgbc_tuning& t, int64_t k, double* bc_dev, int reps,
                 double* ms_out) {
  g->tune = t;
  LGBC_TRY(ensure_hubs(g));
  double best = 1e300;
  for (int r = 0; r <= reps; ++r) {
    LGBC_CUDA(cudaEventRecord(g->ev_start, g->stream));
    LGBC_TRY(run_betweenness(g, k, 0, bc_dev));
    LGBC_CUDA(cudaEventRecord(g->ev_stop, g->stream));
    LGBC_CUDA(cudaEventSynchronize(g->ev_stop));
    float ms = 0.f;
    LGBC_CUDA(cudaEventElapsedTime(&ms, g->ev_start, g->ev_stop));
    if (r > 0) best = std::min(best, static_cast<double>(ms));
  }
  *ms_out = best;
  return LGBC_OK;
}

}  // namespace

extern "C" int lgbc_tune(lgbc_graph* g, const char* cache_path) {
  LGBC_TRY(check_graph(g));
  std::lock_guard<std::mutex> lock(g->mu);
  LGBC_TRY(use_device(g));
  reset_stats(g);
  const std::string sig = tune_signature(g);
  lgbc_tuning cached{};
  if (tune_from_cache(cache_path, sig, &cached)) {
    g->tune = cached;
    return LGBC_OK;
  }
  // sample: 128 active sources spread evenly over the vertex ids
  std::vector<int32_t> act;
  for (int64_t v = 0; v < g->n; ++v)
    if (g->has_degree[static_cast<size_t>(v)]) act.push_back(static_cast<int32_t>(v));
  if (act.empty()) return LGBC_OK;  // nothing to traverse: keep the defaults
  const int64_t k = std::min<int64_t>(128, static_cast<int64_t>(act.size()));
  std::vector<int32_t> sample(static_cast<size_t>(k));
  for (int64_t i = 0; i < k; ++i)
    sample[static_cast<size_t>(i)] = act[static_cast<size_t>(i * static_cast<int64_t>(act.size()) / k)];
  LGBC_TRY(ensure_src(g, k));
  g->h_active = sample;
  g->h_weights.clear();
  LGBC_CUDA(cudaMemcpyAsync(g->d_src, sample.data(), static_cast<size_t>(k) * 4,
                            cudaMemcpyHostToDevice, g->stream));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  LGBC_TRY(ensure_ms(g, true));
  if (!g->d_bc) LGBC_TRY(dev_alloc(&g->d_bc, static_cast<size_t>(g->n)));
  // coordinate descent over the degree-bin cut, the batch width, the
  // direction-switch thresholds and the two gather-strategy cuts
  lgbc_tuning best = g->tune;
  double best_ms = 0.0;
  LGBC_TRY(tune_measure(g, best, k, g->d_bc, 2, &best_ms));
  const int reps = 2;
  for (int pass = 0; pass < 2; ++pass) {
    auto try_field = [&](auto setter, const auto& values) -> int {
      for (const auto& val : values) {
        lgbc_tuning c = best;
        setter(c, val);
        if (std::memcmp(&c, &best, sizeof c) == 0) continue;
        double ms = 0.0;
        LGBC_TRY(tune_measure(g, c, k, g->d_bc, reps, &ms));
        if (ms < best_ms * 0.98) {  // a change must win by 2 %
          best = c;
          best_ms = ms;
        }
      }
      return LGBC_OK;
    };
    const int hubs[] = {64, 128, 256, 512, 1024, 4096, INT32_MAX};
    const int lanes[] = {32, 48, 64};
    const double alphas[] = {2.0, 4.0, 8.0, 14.0, 24.0, 48.0};
    const double betas[] = {6.0, 12.0, 24.0, 48.0, 96.0};
    const int dense[] = {4, 8, 16, 32};
    const int segs[] = {0, 1 << 30};
    LGBC_TRY(try_field([](lgbc_tuning& c, int v) { c.hub_degree = v; }, hubs));
    LGBC_TRY(try_field([](lgbc_tuning& c, int v) { c.lanes = v; }, lanes));
    LGBC_TRY(try_field([](lgbc_tuning& c, double v) { c.alpha = v; }, alphas));
    LGBC_TRY(try_field([](lgbc_tuning& c, double v) { c.beta = v; }, betas));
    LGBC_TRY(try_field([](lgbc_tuning& c, int v) { c.dense_edges = v; }, dense));
    LGBC_TRY(try_field([](lgbc_tuning& c, int v) { c.segment_degree = v; }, segs));
  }
  g->tune = best;
  LGBC_TRY(ensure_hubs(g));
  if (cache_path) {
    FILE* f = std::fopen(cache_path, "a");
    if (!f) return fail(LGBC_EINVAL, std::string("cannot append to tuning cache ") + cache_path);
    std::fprintf(f, "%s %.17g %.17g %d %d %d %d %d %d %d\n", sig.c_str(), best.alpha, best.beta,
                 best.hub_degree, best.lanes, best.dense_edges, best.segment_degree,
                 best.source_order, best.graph_loop, best.stack_vertices);
    std::fclose(f);
  }
  finish_stats(g);
  return LGBC_OK;
}

// ---------------------------------------------------------------------------
// Stress centrality
// ---------------------------------------------------------------------------
extern "C" int lgbc_stress(lgbc_graph* g, const int32_t* src, int64_t nsrc, int64_t* stress_out) {
  LGBC_TRY(check_graph(g));
  std::lock_guard<std::mutex> lock(g->mu);
  LGBC_TRY(use_device(g));
  if (!stress_out && g->n > 0) return fail(LGBC_EINVAL, "null output");
  reset_stats(g);
  int64_t k_act = 0;
  LGBC_TRY(prepare_sources(g, src, nsrc, &k_act));
  g->stats.active_sources = k_act;
  if (g->n == 0) return LGBC_OK;
  unsigned long long* d_st = nullptr;
  LGBC_TRY(dev_alloc(&d_st, static_cast<size_t>(g->n)));
  std::unique_ptr<unsigned long long, void (*)(unsigned long long*)> guard(
      d_st, [](unsigned long long* q) { cudaFree(q); });
  LGBC_CUDA(cudaMemsetAsync(d_st, 0, static_cast<size_t>(g->n) * 8, g->stream));
  if (k_act > 0) LGBC_TRY(ensure_ms(g, true));  // the path-count rows hold E
  for (int64_t s0 = 0; s0 < k_act; s0 += kMaxLanes) {
    const int nl = static_cast<int>(std::min<int64_t>(kMaxLanes, k_act - s0));
    LGBC_TRY(run_ms_batch(g, g->d_src + s0, nl, kSigmaNone, nullptr, nullptr, 0, Seeds(), nullptr,
                          nullptr, d_st));
    g->stats.batches++;
  }
  LGBC_CUDA(cudaMemcpyAsync(stress_out, d_st, static_cast<size_t>(g->n) * 8, cudaMemcpyDeviceToHost,
                            g->stream));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  finish_stats(g);
  return LGBC_OK;
}

// ---------------------------------------------------------------------------
// BFS parents and reachability
// ---------------------------------------------------------------------------
extern "C" int lgbc_bfs_parents(lgbc_graph* g, int32_t s, int dir, int32_t* parents_out) {
  LGBC_TRY(check_graph(g));
  std::lock_guard<std::mutex> lock(g->mu);
  LGBC_TRY(use_device(g));
  if (dir != 0 && dir != 1) return fail(LGBC_EINVAL, "dir must be 0 (out) or 1 (in)");
  if (!parents_out && g->n > 0) return fail(LGBC_EINVAL, "null output");
  LGBC_TRY(check_sources(g, &s, 1));
  reset_stats(g);
  DevGraph dg = g->dev();
  if (dir == 1) {  // follow in-edges: swap the two CSRs
    std::swap(dg.rowptr, dg.in_rowptr);
    std::swap(dg.colidx, dg.in_colidx);
  }
  LGBC_TRY(prepare_bfs(g, &s, 1));
  LGBC_TRY(run_bfs(g, dg, 1));
  int32_t* d_par = nullptr;
  LGBC_TRY(dev_alloc(&d_par, static_cast<size_t>(g->n)));
  std::unique_ptr<int32_t, void (*)(int32_t*)> guard(d_par, [](int32_t* q) { cudaFree(q); });
  g->launches += bfs_parents(g->cfg, g->stream, dg, g->d_dist, d_par);
  LGBC_TRY(check_launch(g));
  LGBC_CUDA(cudaMemcpyAsync(parents_out, d_par, static_cast<size_t>(g->n) * 4,
                            cudaMemcpyDeviceToHost, g->stream));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  finish_stats(g);
  return LGBC_OK;
}

extern "C" int lgbc_has_path(lgbc_graph* g, int32_t u, int32_t v, const int32_t* exclude,
                             int64_t nexclude, int* result) {
  LGBC_TRY(check_graph(g));
  std::lock_guard<std::mutex> lock(g->mu);
  LGBC_TRY(use_device(g));
  if (!result) return fail(LGBC_EINVAL, "null output");
  LGBC_TRY(check_sources(g, &u, 1));
  LGBC_TRY(check_sources(g, &v, 1));
  LGBC_TRY(check_sources(g, exclude, nexclude));
  reset_stats(g);
  for (int64_t i = 0; i < nexclude; ++i)
    if (exclude[i] == u || exclude[i] == v) {
      *result = 0;
      return LGBC_OK;
    }
  if (u == v) {
    *result = 1;
    return LGBC_OK;
  }
  LGBC_TRY(prepare_bfs(g, &u, 1));
  int32_t* d_ex = nullptr;
  if (nexclude > 0) {
    // excluded vertices count as visited from the start (a distance the BFS
    // never writes), so the search neither claims nor expands them
    LGBC_TRY(dev_alloc(&d_ex, static_cast<size_t>(nexclude)));
    LGBC_CUDA(cudaMemcpyAsync(d_ex, exclude, static_cast<size_t>(nexclude) * 4,
                              cudaMemcpyHostToDevice, g->stream));
    g->launches += scatter_i32(g->cfg, g->stream, g->d_dist, d_ex, nexclude, -2);
  }
  std::unique_ptr<int32_t, void (*)(int32_t*)> guard(d_ex, [](int32_t* q) { if (q) cudaFree(q); });
  LGBC_TRY(run_bfs(g, g->dev(), 1));
  int32_t dv = kUnreached;
  LGBC_CUDA(cudaMemcpyAsync(&dv, g->d_dist + v, 4, cudaMemcpyDeviceToHost, g->stream));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  *result = dv != kUnreached ? 1 : 0;
  finish_stats(g);
  return LGBC_OK;
}

// ---------------------------------------------------------------------------
// Graph ingest on the device (ingest.cu)
// ---------------------------------------------------------------------------
namespace {

// Sort `count` keys (owned: keys / alt swap), keep the first copy of each, and
// emit the CSR rows into colidx (allocated here) and rowptr.  With `sorted_out`
// the kept keys are also returned compacted.
int build_rows(lgbc_graph* g, unsigned long long*& keys, unsigned long long*& alt, int64_t count,
               int B, int32_t** colidx, int64_t* rowptr_dev, int64_t* nnz,
               unsigned long long** sorted_out) {
  cudaStream_t s = g->stream;
  const int64_t cells = radix_scratch_words(count);
  const int64_t nsums = std::max<int64_t>(std::max(scan_tiles(cells), scan_tiles(count)),
                                          scan_tiles(g->n)) + 1;
  uint32_t* hist = nullptr;
  int64_t* off = nullptr;
  int64_t* sums = nullptr;
  uint8_t* keep = nullptr;
  int64_t* pos = nullptr;
  unsigned int* deg = nullptr;
  int64_t* d_nkept = nullptr;
  auto cleanup = [&]() {
    cudaFree(hist); cudaFree(off); cudaFree(sums); cudaFree(keep); cudaFree(pos); cudaFree(deg);
    cudaFree(d_nkept);
  };
  int rc = LGBC_OK;
  if ((rc = dev_alloc(&hist, static_cast<size_t>(cells))) || (rc = dev_alloc(&off, static_cast<size_t>(cells))) ||
      (rc = dev_alloc(&sums, static_cast<size_t>(nsums))) || (rc = dev_alloc(&keep, static_cast<size_t>(count))) ||
      (rc = dev_alloc(&pos, static_cast<size_t>(count))) || (rc = dev_alloc(&deg, static_cast<size_t>(g->n))) ||
      (rc = dev_alloc(&d_nkept, 1))) {
    cleanup();
    return rc;
  }
  g->launches += radix_sort(s, keys, alt, count, 2 * B, hist, off, sums);
  g->launches += ingest_unique(g->cfg, s, keys, count, keep, pos, sums, d_nkept);
  int64_t nk = 0;
  cudaError_t e = cudaMemcpyAsync(&nk, d_nkept, 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    cleanup();
    return cuda_fail(e, "ingest: unique arcs");
  }
  if (count == 0) nk = 0;
  *nnz = nk;
  if ((rc = dev_alloc(colidx, static_cast<size_t>(std::max<int64_t>(nk, 1))))) {
    cleanup();
    return rc;
  }
  cudaMemsetAsync(deg, 0, static_cast<size_t>(g->n) * 4, s);
  g->launches += ingest_emit(g->cfg, s, keys, count, keep, pos, B, *colidx, deg);
  g->launches += ingest_rowptr(s, deg, g->n, sums, rowptr_dev);
  if (g->n == 0) cudaMemsetAsync(rowptr_dev, 0, 8, s);
  if (sorted_out) {
    *sorted_out = alt;  // reuse the spare buffer for the compacted keys
    alt = nullptr;
    g->launches += ingest_compact(g->cfg, s, keys, count, keep, pos, *sorted_out);
  }
  e = cudaStreamSynchronize(s);
  cleanup();
  if (e != cudaSuccess) return cuda_fail(e, "ingest: rows");
  return check_launch(g);
}

int create_from_edges_impl(lgbc_graph* g, int64_t n, int64_t m, const int32_t* src,
                           const int32_t* dst, int directed) {
  LGBC_TRY(init_handle(g, n, directed));
  cudaStream_t s = g->stream;
  const int B = ingest_bits(n);
  const int64_t count = directed ? m : 2 * m;
  int32_t* d_edges = nullptr;
  unsigned long long* keys = nullptr;
  unsigned long long* alt = nullptr;
  int* d_bad = nullptr;
  auto cleanup = [&]() { cudaFree(d_edges); cudaFree(keys); cudaFree(alt); cudaFree(d_bad); };
  int rc = LGBC_OK;
  if ((rc = dev_alloc(&d_edges, static_cast<size_t>(2 * std::max<int64_t>(m, 1)))) ||
      (rc = dev_alloc(&keys, static_cast<size_t>(std::max<int64_t>(count, 1)))) ||
      (rc = dev_alloc(&alt, static_cast<size_t>(std::max<int64_t>(count, 1)))) ||
      (rc = dev_alloc(&d_bad, 1))) {
    cleanup();
    return rc;
  }
  cudaMemsetAsync(d_bad, 0, 4, s);
  if (m > 0) {
    LGBC_CUDA(cudaMemcpyAsync(d_edges, src, static_cast<size_t>(m) * 4, cudaMemcpyHostToDevice, s));
    LGBC_CUDA(cudaMemcpyAsync(d_edges + m, dst, static_cast<size_t>(m) * 4, cudaMemcpyHostToDevice, s));
  }
  g->launches += ingest_make_keys(g->cfg, s, d_edges, d_edges + m, m, n, B, directed, keys, d_bad);
  int bad = 0;
  LGBC_CUDA(cudaMemcpyAsync(&bad, d_bad, 4, cudaMemcpyDeviceToHost, s));
  LGBC_CUDA(cudaStreamSynchronize(s));
  if (bad) {
    cleanup();
    return fail(LGBC_EINVAL, "edge endpoint outside [0, n)");
  }
  cudaFree(d_edges);
  d_edges = nullptr;
  if ((rc = dev_alloc(&g->d_rowptr, static_cast<size_t>(n + 1)))) {
    cleanup();
    return rc;
  }
  unsigned long long* sorted = nullptr;
  int64_t nnz = 0;
  rc = build_rows(g, keys, alt, count, B, &g->d_colidx, g->d_rowptr, &nnz, directed ? &sorted : nullptr);
  if (rc != LGBC_OK) {
    cudaFree(sorted);
    cleanup();
    return rc;
  }
  g->nnz = nnz;
  std::vector<int64_t> rp(static_cast<size_t>(n + 1)), irp;
  if (directed) {
    // in-CSR: the kept arcs with their ends swapped, sorted again
    cudaFree(keys);
    keys = nullptr;
    unsigned long long* ikeys = nullptr;
    if ((rc = dev_alloc(&ikeys, static_cast<size_t>(std::max<int64_t>(nnz, 1))))) {
      cudaFree(sorted);
      cleanup();
      return rc;
    }
    g->launches += ingest_swap_keys(g->cfg, s, sorted, nnz, B, ikeys);
    unsigned long long* ialt = sorted;
    if ((rc = dev_alloc(&g->d_in_rowptr, static_cast<size_t>(n + 1)))) {
      cudaFree(ikeys);
      cudaFree(ialt);
      cleanup();
      return rc;
    }
    int64_t innz = 0;
    rc = build_rows(g, ikeys, ialt, nnz, B, &g->d_in_colidx, g->d_in_rowptr, &innz, nullptr);
    cudaFree(ikeys);
    cudaFree(ialt);
    if (rc != LGBC_OK) {
      cleanup();
      return rc;
    }
    irp.resize(static_cast<size_t>(n + 1));
    LGBC_CUDA(cudaMemcpy(irp.data(), g->d_in_rowptr, irp.size() * 8, cudaMemcpyDeviceToHost));
  } else {
    g->d_in_rowptr = g->d_rowptr;
    g->d_in_colidx = g->d_colidx;
  }
  cleanup();
  LGBC_CUDA(cudaMemcpy(rp.data(), g->d_rowptr, rp.size() * 8, cudaMemcpyDeviceToHost));
  return finish_handle(g, rp.data(), directed ? irp.data() : rp.data());
}

}  // namespace

extern "C" int lgbc_graph_create_from_edges(lgbc_graph** out, int64_t n, int64_t m,
                                            const int32_t* src, const int32_t* dst, int directed) {
  if (!out) return fail(LGBC_EINVAL, "null output handle pointer");
  *out = nullptr;
  if (n < 0 || m < 0) return fail(LGBC_EINVAL, "negative vertex or edge count");
  if (n >= INT32_MAX) return fail(LGBC_EINVAL, "vertex ids must fit in int32");
  if (m > 0 && (!src || !dst)) return fail(LGBC_EINVAL, "null edge array");
  if (m > (int64_t{1} << 31) - 1) return fail(LGBC_EINVAL, "at most 2^31 - 1 edges per call");
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(LGBC_ECUDA, std::string("no CUDA device available: ") +
                                (e != cudaSuccess ? cudaGetErrorString(e) : "0 devices"));
  }
  lgbc_graph* g = new (std::nothrow) lgbc_graph();
  if (!g) return fail(LGBC_ENOMEM, "host allocation failed");
  const int rc = create_from_edges_impl(g, n, m, src, dst, directed);
  if (rc != LGBC_OK) {
    const std::string msg = g_last_error;
    lgbc_graph_destroy(g);
    g_last_error = msg;
    return rc;
  }
  *out = g;
  return LGBC_OK;
}

extern "C" int lgbc_graph_csr(const lgbc_graph* g, int64_t* rowptr, int32_t* colidx,
                              int64_t* in_rowptr, int32_t* in_colidx) {
  LGBC_TRY(check_graph(g));
  lgbc_graph* gm = const_cast<lgbc_graph*>(g);
  std::lock_guard<std::mutex> lock(gm->mu);
  LGBC_TRY(use_device(gm));
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  if (rowptr)
    LGBC_CUDA(cudaMemcpy(rowptr, g->d_rowptr, static_cast<size_t>(g->n + 1) * 8, cudaMemcpyDeviceToHost));
  if (colidx && g->nnz > 0)
    LGBC_CUDA(cudaMemcpy(colidx, g->d_colidx, static_cast<size_t>(g->nnz) * 4, cudaMemcpyDeviceToHost));
  if (in_rowptr)
    LGBC_CUDA(cudaMemcpy(in_rowptr, g->d_in_rowptr, static_cast<size_t>(g->n + 1) * 8,
                         cudaMemcpyDeviceToHost));
  if (in_colidx && g->nnz > 0)
    LGBC_CUDA(cudaMemcpy(in_colidx, g->d_in_colidx, static_cast<size_t>(g->nnz) * 4,
                         cudaMemcpyDeviceToHost));
  return LGBC_OK;
}
