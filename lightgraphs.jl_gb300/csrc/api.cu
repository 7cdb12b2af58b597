// api.cu -- the C ABI of include/lgbc.h: graph handles, workspaces and the
// host side of the level loops.  All arithmetic runs in the kernels of
// msbfs.cu / bfs.cu / util.cu; there is no CPU fallback.  The other entry
// points live in api_many.cu, api_learned.cu and api_more.cu.
#include "api_internal.h"

using namespace lgbc;
using namespace lgbc::api;

// Lets the other translation units of the library report errors through
// lgbc_last_error().
void lgbc::set_last_error(const char* msg) { g_last_error = msg ? msg : ""; }

namespace lgbc::api {

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

int ensure_ms(lgbc_graph* g, bool need_sigma, int words) {
  MsWorkspace& w = g->ms;
  const size_t n = static_cast<size_t>(g->n);
  const size_t mask_words = n * kMaxWords;
  if (!w.visit) {
    LGBC_TRY(dev_alloc(&w.visit, mask_words));
    LGBC_TRY(dev_alloc(&w.mb0, mask_words));
    LGBC_TRY(dev_alloc(&w.mb1, mask_words));
    LGBC_TRY(dev_alloc(&w.lvl_off, n + 3));
    LGBC_TRY(dev_alloc(&w.ctl, 1));
    LGBC_CUDA(cudaMemsetAsync(w.visit, 0, mask_words * 8, g->stream));
    LGBC_CUDA(cudaMemsetAsync(w.mb0, 0, mask_words * 8, g->stream));
    LGBC_CUDA(cudaMemsetAsync(w.mb1, 0, mask_words * 8, g->stream));
  }
  if (!w.qv) {
    const unsigned long long cap = 4ull * n + 1024;
    LGBC_TRY(dev_alloc(&w.qv, cap));
    LGBC_TRY(dev_alloc(&w.qm, cap * kMaxWords));
    w.cap = cap;
  }
  if (words > 1 && !w.claim) {
    LGBC_TRY(dev_alloc(&w.claim, n + 1));
    LGBC_CUDA(cudaMemsetAsync(w.claim, 0, (n + 1) * sizeof(unsigned), g->stream));
  }
  if (need_sigma && w.sigma_words < words) {
    LGBC_CUDA(cudaStreamSynchronize(g->stream));
    if (w.sigma) cudaFree(w.sigma);
    if (w.psi) cudaFree(w.psi);
    w.sigma = w.psi = nullptr;
    w.sigma_words = 0;
    const size_t row = static_cast<size_t>(64) * static_cast<size_t>(words);
    unsigned long long* s = nullptr;
    unsigned long long* p = nullptr;
    LGBC_TRY(dev_alloc(&s, n * row));
    int rc = dev_alloc(&p, n * row);
    if (rc != LGBC_OK) {
      cudaFree(s);
      return rc;
    }
    w.sigma = s;
    w.psi = p;
    w.sigma_words = words;
  }
  return LGBC_OK;
}

int grow_ms_lists(lgbc_graph* g) {
  MsWorkspace& w = g->ms;
  const unsigned long long n = static_cast<unsigned long long>(g->n);
  // every lane puts a vertex on at most one level: lanes x n entries + level 0
  const unsigned long long max_cap = (kWideLanes + 1ull) * n + 1024;
  unsigned long long cap = std::min(max_cap, w.cap * 2);
  if (cap <= w.cap) return fail(LGBC_ENOMEM, "level lists cannot grow further");
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  dev_free(w.qv);
  dev_free(w.qm);
  LGBC_TRY(dev_alloc(&w.qv, cap));
  LGBC_TRY(dev_alloc(&w.qm, cap * kMaxWords));
  w.cap = cap;
  return LGBC_OK;
}

int ensure_bfs(lgbc_graph* g) {
  BfsWorkspace& w = g->bfs;
  if (w.queue) return LGBC_OK;
  const size_t n = static_cast<size_t>(g->n);
  const size_t words = (n + 31) / 32 + 4;
  LGBC_TRY(dev_alloc(&w.queue, n + 1));
  LGBC_TRY(dev_alloc(&w.large, n + 1));
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

// Cut every edge list longer than H into kHubChunk-edge work items, in the
// order `order` selects: 0 hub by hub; 1 by the neighbour id of each item's
// middle edge (colidx must be given); 2 by the relative position of each
// item's middle in its hub's row (on rows sorted by neighbour id this follows
// order 1 without reading colidx).  Orders 1 and 2 interleave the hubs: the
// grid works through the item list roughly in order, so the items in flight
// at one time gather rows of a limited range of vertices (reused from L2 by
// the hubs that share them) and a hub's items are spread out (fewer
// simultaneous atomics on one accumulator row).  Any order gives the same
// results.
void make_items(const int64_t* rowptr, const int32_t* colidx, int64_t n, int H, int order,
                const std::vector<int32_t>& slot_of, std::vector<HubItem>& items) {
  constexpr int64_t kBuckets = int64_t(1) << 16;
  const bool ordered = order == 2 || (order == 1 && colidx != nullptr && n > 0);
  // items (and their order keys) per contiguous part of the vertex range,
  // concatenated in vertex order
  std::vector<std::vector<HubItem>> pit(8);
  std::vector<std::vector<int64_t>> pkey(8);
  const int parts = parallel_parts(n, [&](int p, int64_t vb, int64_t ve) {
    std::vector<HubItem>& out = pit[static_cast<size_t>(p)];
    std::vector<int64_t>& key = pkey[static_cast<size_t>(p)];
    for (int64_t v = vb; v < ve; ++v) {
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
        out.push_back(it);
        if (!ordered) continue;
        const int64_t mid2 = (lo - e0) + it.hi - e0;  // twice the middle's offset in the row
        key.push_back(order == 1 ? static_cast<int64_t>(colidx[lo + (it.hi - lo) / 2]) * kBuckets / n
                                 : mid2 * kBuckets / (2 * (e1 - e0)));
      }
    }
  });
  items.clear();
  std::vector<int64_t> key;
  for (int p = 0; p < parts; ++p) {
    items.insert(items.end(), pit[static_cast<size_t>(p)].begin(), pit[static_cast<size_t>(p)].end());
    key.insert(key.end(), pkey[static_cast<size_t>(p)].begin(), pkey[static_cast<size_t>(p)].end());
  }
  if (!ordered) return;
  // stable counting sort on the bucket
  std::vector<int64_t> start(static_cast<size_t>(kBuckets + 1), 0);
  for (int64_t k : key) start[static_cast<size_t>(k + 1)]++;
  for (int64_t bk = 0; bk < kBuckets; ++bk) start[static_cast<size_t>(bk + 1)] += start[static_cast<size_t>(bk)];
  std::vector<HubItem> sorted(items.size());
  for (size_t i = 0; i < items.size(); ++i) sorted[static_cast<size_t>(start[static_cast<size_t>(key[i])]++)] = items[i];
  items.swap(sorted);
}

int upload_items(const std::vector<HubItem>& items, HubItem** out) {
  *out = nullptr;
  if (items.empty()) return LGBC_OK;
  LGBC_TRY(dev_alloc(out, items.size()));
  LGBC_CUDA(cudaMemcpy(*out, items.data(), items.size() * sizeof(HubItem), cudaMemcpyHostToDevice));
  return LGBC_OK;
}

// Build the hub work items from host copies of rowptr / in_rowptr; colidx /
// in_colidx are host copies or null (then copied from the device when item
// order 1 needs them).
int build_hubs(lgbc_graph* g, const int64_t* rowptr, const int32_t* colidx, const int64_t* in_rowptr,
               const int32_t* in_colidx, int H, int order) {
  g->hubs.release();
  const int64_t n = g->n;
  std::vector<int32_t> slot_of(static_cast<size_t>(n), -1);
  auto is_hub = [&](int64_t v) {
    return rowptr[v + 1] - rowptr[v] > H || in_rowptr[v + 1] - in_rowptr[v] > H;
  };
  // slots in vertex order: count per part, then number
  std::vector<int64_t> first(9, 0);
  const int parts = parallel_parts(n, [&](int p, int64_t vb, int64_t ve) {
    int64_t c = 0;
    for (int64_t v = vb; v < ve; ++v) c += is_hub(v) ? 1 : 0;
    first[static_cast<size_t>(p + 1)] = c;
  });
  for (int p = 0; p < parts; ++p) first[static_cast<size_t>(p + 1)] += first[static_cast<size_t>(p)];
  const int64_t nslots = first[static_cast<size_t>(parts)];
  parallel_parts(n, [&](int p, int64_t vb, int64_t ve) {
    int64_t next = first[static_cast<size_t>(p)];
    for (int64_t v = vb; v < ve; ++v)
      if (is_hub(v)) slot_of[static_cast<size_t>(v)] = static_cast<int32_t>(next++);
  });
  g->hubs.nslots = nslots;
  g->hubs.built_for = H;
  g->hubs.built_order = order;
  if (nslots == 0) return LGBC_OK;
  std::vector<int32_t> ci, ici;
  if (order == 1 && g->nnz > 0) {
    if (!colidx) {
      LGBC_CUDA(cudaStreamSynchronize(g->stream));
      ci.resize(static_cast<size_t>(g->nnz));
      LGBC_CUDA(cudaMemcpy(ci.data(), g->d_colidx, ci.size() * 4, cudaMemcpyDeviceToHost));
      colidx = ci.data();
    }
    if (g->directed && !in_colidx) {
      ici.resize(static_cast<size_t>(g->nnz));
      LGBC_CUDA(cudaMemcpy(ici.data(), g->d_in_colidx, ici.size() * 4, cudaMemcpyDeviceToHost));
      in_colidx = ici.data();
    }
  }
  std::vector<HubItem> items;
  make_items(rowptr, colidx, n, H, order, slot_of, items);
  g->hubs.n_out = static_cast<int64_t>(items.size());
  LGBC_TRY(upload_items(items, &g->hubs.out_items));
  if (g->directed) {
    make_items(in_rowptr, in_colidx, n, H, order, slot_of, items);
    g->hubs.n_in = static_cast<int64_t>(items.size());
    LGBC_TRY(upload_items(items, &g->hubs.in_items));
  } else {
    g->hubs.in_items = g->hubs.out_items;
    g->hubs.n_in = g->hubs.n_out;
  }
  // accumulators for the widest batch: 64 * kMaxWords lanes, kMaxWords mask words
  LGBC_TRY(dev_alloc(&g->hubs.acc, static_cast<size_t>(nslots) * kWideLanes));
  LGBC_TRY(dev_alloc(&g->hubs.mask, static_cast<size_t>(nslots) * kMaxWords));
  LGBC_TRY(dev_alloc(&g->hubs.cnt, static_cast<size_t>(nslots)));
  LGBC_CUDA(cudaMemset(g->hubs.acc, 0, static_cast<size_t>(nslots) * kWideLanes * 8));
  LGBC_CUDA(cudaMemset(g->hubs.mask, 0, static_cast<size_t>(nslots) * kMaxWords * 8));
  LGBC_CUDA(cudaMemset(g->hubs.cnt, 0, static_cast<size_t>(nslots) * 4));
  return LGBC_OK;
}

// Rebuild the hub table after hub_degree or hub_order changed (rowptr copied back).
int ensure_hubs(lgbc_graph* g) {
  if (g->hubs.built_for == g->tune.hub_degree && g->hubs.built_order == g->tune.hub_order)
    return LGBC_OK;
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  std::vector<int64_t> rp(static_cast<size_t>(g->n + 1)), irp;
  LGBC_CUDA(cudaMemcpy(rp.data(), g->d_rowptr, rp.size() * 8, cudaMemcpyDeviceToHost));
  const int64_t* in_rp = rp.data();
  if (g->directed) {
    irp.resize(rp.size());
    LGBC_CUDA(cudaMemcpy(irp.data(), g->d_in_rowptr, irp.size() * 8, cudaMemcpyDeviceToHost));
    in_rp = irp.data();
  }
  return build_hubs(g, rp.data(), nullptr, in_rp, nullptr, g->tune.hub_degree, g->tune.hub_order);
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

MsBuffers ms_buffers(lgbc_graph* g, const int32_t* lane_src, const double* lane_w) {
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
  b.claim = w.claim;
  b.words = 1;
  // lanes die at reachability boundaries in digraphs (every vertex a source
  // cannot reach); on undirected graphs with one giant component the filter
  // costs more than it skips
  b.lane_filter = g->directed ? 1 : 0;
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

LoopKey loop_key(lgbc_graph* g, int backward, int sigma_kind, const LaneSet& act,
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
                 int32_t* dist, int64_t dist_ld, const Seeds& seeds, const double* lane_w,
                 const LevelStats* stats, unsigned long long* stress, const PathExport* pexp) {
  const DevGraph dg = g->dev();
  LGBC_TRY(ensure_hubs(g));
  const HubData hd = hub_data(g);
  // more than 64 lanes: a two- or four-word batch (Brandes batches only)
  const int words = lane_words(nl);
  if (nl < 1 || nl > kWideLanes)
    return fail(LGBC_EINVAL, "internal: a multi-source batch holds 1 to 256 lanes");
  if (words > 1 && (dist || stats || stress || pexp || sigma_kind == kSigmaNone ||
                    g->ms.sigma_words < words || !g->ms.claim))
    return fail(LGBC_EINVAL, "internal: a multi-word batch is a Brandes batch");
  if (pexp && (sigma_kind == kSigmaNone || seeds.v))
    return fail(LGBC_EINVAL, "internal: a path-count export needs a plain batch with path counts");
  // a W-word lane set is read as one aligned 8 W-byte access
  auto misaligned = [&](const void* p) {
    return words > 1 && (reinterpret_cast<uintptr_t>(p) & (8u * words - 1u)) != 0;
  };
  if (misaligned(seeds.mask) || misaligned(seeds.seg_mark))
    return fail(LGBC_EINVAL, "internal: seed lane sets must be aligned to their size");
  const LaneSet act = lane_set(nl, words);
  for (;;) {
    MsBuffers b = ms_buffers(g, lane_src, lane_w);
    b.words = words;
    b.lane_w_n = seeds.lane_w_n;
    if (seeds.seg_mark) g->launches += ms_premark(g->cfg, g->stream, b, seeds.seg_off, seeds.seg_mark,
                                                  seeds.nseg);
    if (seeds.v)
      g->launches += ms_init_seeds(g->cfg, g->stream, dg, b, seeds.v, seeds.mask, seeds.count,
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
      if (c.overflow_sigma && u64_counts(sigma_kind)) {
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
      if (pexp) {
        g->launches += ms_export(g->cfg, g->stream, b, sigma_kind, pexp->sigma, pexp->dist, pexp->ld);
        g->launches += ms_cleanup_all(g->cfg, g->stream, b);
        return check_launch(g);
      }
      const int maxl = c.maxlevel;
      LoopGraph* bg = nullptr;
      LGBC_TRY(get_loop(g, loop_key(g, 1, sigma_kind, act, nullptr, 0, bc, bw, hd), &bg));
      LGBC_CUDA(cudaGraphLaunch(bg->exec, g->stream));
      g->launches += 2 + static_cast<int64_t>(maxl + 1) * bg->body_kernels;
      if (seeds.seg_mark)  // premarked vertices were never listed: clear visit outright
        LGBC_CUDA(cudaMemsetAsync(b.visit, 0, static_cast<size_t>(g->n) * 8 * words, g->stream));
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
      if (c.overflow_sigma && u64_counts(sigma_kind)) break;
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
    if (g->h_ctl->overflow_sigma && u64_counts(sigma_kind)) {
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
    if (pexp) {
      g->launches += ms_export(g->cfg, g->stream, b, sigma_kind, pexp->sigma, pexp->dist, pexp->ld);
      g->launches += ms_cleanup_all(g->cfg, g->stream, b);
      return check_launch(g);
    }
    const int maxl = g->h_ctl->maxlevel;
    g->launches += ms_begin_backward(g->stream, b);
    for (int L = maxl; L >= 0; --L)
      g->launches += ms_backward_level(g->cfg, g->stream, dg, b, hd, sigma_kind, bc);
    g->launches += ms_cleanup(g->cfg, g->stream, b);
    if (seeds.seg_mark)  // premarked vertices were never listed: clear visit outright
      LGBC_CUDA(cudaMemsetAsync(b.visit, 0, static_cast<size_t>(g->n) * 8 * words, g->stream));
    return check_launch(g);
  }
}

// Brandes over the active sources already on the device (g->d_src[0, k)),
// accumulating into bc_dev (zeroed here); with d_w, source i's dependencies
// are scaled by d_w[i].
int run_stacked(lgbc_graph* g, int64_t copies, double* bc_dev, const std::vector<double>* w);

int run_betweenness(lgbc_graph* g, int64_t k_act, int endpoints, double* bc_dev,
                    const double* d_w) {
  g->launches += fill_f64(g->cfg, g->stream, bc_dev, g->n, 0.0);
  const int lanes0 = std::max(1, std::min<int>(kWideLanes, g->tune.lanes));
  const int64_t batches = (k_act + lanes0 - 1) / lanes0;
  const int64_t copies = g->n > 0 ? std::min<int64_t>(g->tune.stack_vertices / g->n, batches) : 0;
  const bool host_w = d_w && static_cast<int64_t>(g->h_weights.size()) == k_act;
  if ((!d_w || host_w) && copies >= 4 && static_cast<int64_t>(g->h_active.size()) == k_act) {
    LGBC_TRY(run_stacked(g, copies, bc_dev, d_w ? &g->h_weights : nullptr));
    if (endpoints) g->launches += add_endpoints(g->cfg, g->stream, bc_dev, g->n, g->d_src, k_act);
    return check_launch(g);
  }
  const int lanes = std::max(1, std::min<int>(kWideLanes, g->tune.lanes));
  if (k_act > 0) LGBC_TRY(ensure_ms(g, true, lane_words(lanes)));
  for (int64_t s0 = 0; s0 < k_act; s0 += lanes) {
    const int nl = static_cast<int>(std::min<int64_t>(lanes, k_act - s0));
    const double* lw = d_w ? d_w + s0 : nullptr;
    int rc = run_ms_batch(g, g->d_src + s0, nl, dep_kind(g), bc_dev, nullptr, 0, Seeds(), lw);
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
// A handle for the disjoint union of `copies` copies of g, built on the
// device from g's CSR (valid by construction, so not validated again).
int create_replicated(lgbc_graph* g, int64_t copies, lgbc_graph** out) {
  *out = nullptr;
  lgbc_graph* st = new (std::nothrow) lgbc_graph();
  if (!st) return fail(LGBC_ENOMEM, "host allocation failed");
  auto build = [&]() -> int {
    const int64_t n = g->n, nnz = g->nnz, N = copies * n, NNZ = copies * nnz;
    LGBC_TRY(init_handle(st, N, g->directed));
    st->nnz = NNZ;
    LGBC_CUDA(cudaStreamSynchronize(g->stream));  // g's CSR is complete
    LGBC_TRY(dev_alloc(&st->d_rowptr, static_cast<size_t>(N + 1)));
    LGBC_TRY(dev_alloc(&st->d_colidx, static_cast<size_t>(std::max<int64_t>(NNZ, 1))));
    st->launches += replicate_csr(st->cfg, st->stream, g->d_rowptr, g->d_colidx, n, nnz, copies,
                                  st->d_rowptr, st->d_colidx);
    std::vector<int64_t> rp(static_cast<size_t>(N + 1)), irp;
    if (g->directed) {
      LGBC_TRY(dev_alloc(&st->d_in_rowptr, static_cast<size_t>(N + 1)));
      LGBC_TRY(dev_alloc(&st->d_in_colidx, static_cast<size_t>(std::max<int64_t>(NNZ, 1))));
      st->launches += replicate_csr(st->cfg, st->stream, g->d_in_rowptr, g->d_in_colidx, n, nnz,
                                    copies, st->d_in_rowptr, st->d_in_colidx);
      irp.resize(rp.size());
      LGBC_CUDA(cudaMemcpyAsync(irp.data(), st->d_in_rowptr, irp.size() * 8, cudaMemcpyDeviceToHost,
                                st->stream));
    } else {
      st->d_in_rowptr = st->d_rowptr;
      st->d_in_colidx = st->d_colidx;
    }
    LGBC_CUDA(cudaMemcpyAsync(rp.data(), st->d_rowptr, rp.size() * 8, cudaMemcpyDeviceToHost,
                              st->stream));
    LGBC_CUDA(cudaStreamSynchronize(st->stream));
    LGBC_TRY(check_launch(st));
    return finish_handle(st, rp.data(), g->directed ? irp.data() : rp.data());
  };
  const int rc = build();
  if (rc != LGBC_OK) {
    const std::string msg = g_last_error;
    lgbc_graph_destroy(st);
    g_last_error = msg;
    return rc;
  }
  *out = st;
  return LGBC_OK;
}

int run_stacked(lgbc_graph* g, int64_t copies, double* bc_dev, const std::vector<double>* w) {
  const int64_t n = g->n;
  const int L = std::max(1, std::min<int>(kWideLanes, g->tune.lanes));
  const int W = lane_words(L);  // lane words per vertex of the union batches
  const int64_t row = 64 * W;            // weights per copy row
  if (!g->stack || g->stack_copies != copies) {
    if (g->stack) lgbc_graph_destroy(g->stack);
    g->stack = nullptr;
    g->stack_copies = 0;
    // the union's CSR(s) are replicated on the device: copy r holds vertices [r n, (r + 1) n)
    if (copies * n >= INT32_MAX) return fail(LGBC_EINVAL, "stacked union exceeds int32 vertex ids");
    lgbc_graph* st = nullptr;
    LGBC_TRY(create_replicated(g, copies, &st));
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
  std::vector<int32_t> sv;
  std::vector<uint64_t> sm;
  std::vector<int64_t> bstart(static_cast<size_t>(nbu + 1), 0), voff(static_cast<size_t>(copies + 1));
  // W words per seed mask and per copy mark
  std::vector<uint64_t> marks(static_cast<size_t>(nbu * copies * W));
  std::vector<int64_t> filled(static_cast<size_t>(nbu), 0);  // ordinary batches per union batch
  // lane weights: row u * copies + r holds copy r's 64 W lanes of union batch u
  std::vector<double> wrows(w ? static_cast<size_t>(nbu * copies * row) : 0, 0.0);
  const LaneSet all = lane_set(L, W);
  for (int64_t r = 0; r <= copies; ++r) voff[static_cast<size_t>(r)] = r * n;
  for (int64_t u = 0; u < nbu; ++u) {
    for (int64_t r = 0; r < copies; ++r) {
      if ((u * copies + r) * L < k) filled[static_cast<size_t>(u)]++;
      LaneSet seeded{};
      const int64_t i0 = (u * copies + r) * L;
      const size_t first = sv.size();  // this copy's seeds: a repeated source is one seed
      for (int l = 0; l < L && i0 + l < k; ++l) {
        const int32_t v = static_cast<int32_t>(r * n + act[static_cast<size_t>(i0 + l)]);
        size_t j = first;
        while (j < sv.size() && sv[j] != v) ++j;
        if (j == sv.size()) {
          sv.push_back(v);
          for (int q = 0; q < W; ++q) sm.push_back(0ull);
        }
        sm[j * W + static_cast<size_t>(l >> 6)] |= 1ull << (l & 63);
        seeded.w[l >> 6] |= 1ull << (l & 63);
        if (w) wrows[static_cast<size_t>((u * copies + r) * row + l)] = (*w)[static_cast<size_t>(i0 + l)];
      }
      for (int q = 0; q < W; ++q)
        marks[static_cast<size_t>((u * copies + r) * W + q)] = all.w[q] & ~seeded.w[q];
    }
    bstart[static_cast<size_t>(u + 1)] = static_cast<int64_t>(sv.size());
  }
  // one device buffer: weight rows | voff | marks | seed masks | seed vertices,
  // each part starting on a 32-byte boundary (a W-word lane set is read as
  // one aligned 8 W-byte access)
  auto up32 = [](size_t x) { return (x + 31) & ~static_cast<size_t>(31); };
  const size_t o_voff = up32(wrows.size() * 8);
  const size_t o_marks = up32(o_voff + voff.size() * 8);
  const size_t o_sm = up32(o_marks + marks.size() * 8);
  const size_t o_sv = up32(o_sm + sm.size() * 8);
  const size_t bytes = o_sv + sv.size() * 4 + 16;
  unsigned char* buf = nullptr;
  LGBC_TRY(dev_alloc(&buf, bytes));
  std::unique_ptr<unsigned char, cudaError_t (*)(void*)> guard(buf, cudaFree);
  double* d_wrows = reinterpret_cast<double*>(buf);
  if (!wrows.empty())
    LGBC_CUDA(cudaMemcpyAsync(d_wrows, wrows.data(), wrows.size() * 8, cudaMemcpyHostToDevice,
                              st->stream));
  int64_t* d_voff = reinterpret_cast<int64_t*>(buf + o_voff);
  uint64_t* d_marks = reinterpret_cast<uint64_t*>(buf + o_marks);
  uint64_t* d_sm = reinterpret_cast<uint64_t*>(buf + o_sm);
  int32_t* d_sv = reinterpret_cast<int32_t*>(buf + o_sv);
  LGBC_CUDA(cudaMemcpyAsync(d_voff, voff.data(), voff.size() * 8, cudaMemcpyHostToDevice, st->stream));
  LGBC_CUDA(cudaMemcpyAsync(d_marks, marks.data(), marks.size() * 8, cudaMemcpyHostToDevice, st->stream));
  LGBC_CUDA(cudaMemcpyAsync(d_sm, sm.data(), sm.size() * 8, cudaMemcpyHostToDevice, st->stream));
  LGBC_CUDA(cudaMemcpyAsync(d_sv, sv.data(), sv.size() * 4, cudaMemcpyHostToDevice, st->stream));
  if (!st->d_bc) LGBC_TRY(dev_alloc(&st->d_bc, static_cast<size_t>(st->n)));
  st->launches += fill_f64(st->cfg, st->stream, st->d_bc, st->n, 0.0);
  LGBC_TRY(ensure_ms(st, true, W));
  // the caller's stream waits for nothing of ours: order the two streams
  LGBC_CUDA(cudaStreamSynchronize(g->stream));
  for (int64_t u = 0; u < nbu; ++u) {
    Seeds sd;
    sd.v = d_sv + bstart[static_cast<size_t>(u)];
    sd.mask = d_sm + bstart[static_cast<size_t>(u)] * W;
    sd.count = bstart[static_cast<size_t>(u + 1)] - bstart[static_cast<size_t>(u)];
    sd.seg_off = d_voff;
    sd.seg_mark = d_marks + static_cast<size_t>(u * copies * W);
    sd.nseg = copies;
    const double* lw = nullptr;
    if (w) {
      lw = d_wrows + u * copies * row;
      sd.lane_w_n = n;
      sd.lane_w_count = copies * row;
    }
    int rc = run_ms_batch(st, nullptr, L, dep_kind(st), st->d_bc, nullptr, 0, sd, lw);
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
int finish_handle(lgbc_graph* g, const int64_t* rowptr, const int64_t* in_rowptr,
                  const int32_t* colidx, const int32_t* in_colidx);
void degree_pass(lgbc_graph* g, const int64_t* rowptr, const int64_t* in_rowptr);

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
  // the degree pass (differences of row pointers only) overlaps the upload;
  // the hub items walk row ranges and wait for the validation
  degree_pass(g, rowptr, directed ? in_rowptr : rowptr);
  cudaError_t e = cudaStreamSynchronize(g->stream);
  cudaFree(d_bad);
  if (e != cudaSuccess) return cuda_fail(e, "graph upload");
  LGBC_TRY(check_launch(g));
  if (bad & 1) return fail(LGBC_EINVAL, "rowptr must be non-decreasing");
  if (bad & 2) return fail(LGBC_EINVAL, "column index out of range");
  if (bad & 4) return fail(LGBC_EINVAL, "rowptr must run from 0 to nnz");
  return build_hubs(g, rowptr, colidx, directed ? in_rowptr : rowptr, directed ? in_colidx : colidx,
                    g->tune.hub_degree, g->tune.hub_order);
}

// degree(g, v) > 0 (in+out for digraphs, src/core.jl:66-67), kept on the
// host; the path-count bound; and the kLandmarks highest-degree vertices (ties:
// smaller id) for source ordering.  Reads the row pointers only.
void degree_pass(lgbc_graph* g, const int64_t* rowptr, const int64_t* in_rowptr) {
  const int64_t n = g->n;
  const int directed = g->directed;
  g->has_degree.assign(static_cast<size_t>(n), 0);
  uint8_t* has = g->has_degree.data();
  std::vector<int64_t> max_in(8, 0);
  std::vector<std::vector<std::pair<int64_t, int32_t>>> tops(8);  // max-heaps of (-degree, id)
  const int parts = parallel_parts(n, [&](int p, int64_t vb, int64_t ve) {
    int64_t mi = 0;
    auto& top = tops[static_cast<size_t>(p)];
    for (int64_t v = vb; v < ve; ++v) {
      const int64_t dout = rowptr[v + 1] - rowptr[v];
      const int64_t din = directed ? in_rowptr[v + 1] - in_rowptr[v] : dout;
      const int64_t d = directed ? dout + din : dout;
      has[v] = d > 0 ? 1 : 0;
      mi = std::max(mi, din);
      if (d <= 0) continue;
      if (top.size() < static_cast<size_t>(kLandmarks)) {
        top.emplace_back(-d, static_cast<int32_t>(v));
        std::push_heap(top.begin(), top.end());
      } else if (-d < top.front().first) {  // a larger degree (equal: the smaller id stays)
        std::pop_heap(top.begin(), top.end());
        top.back() = std::make_pair(-d, static_cast<int32_t>(v));
        std::push_heap(top.begin(), top.end());
      }
    }
    max_in[static_cast<size_t>(p)] = mi;
  });
  int64_t mi = 0;
  std::vector<std::pair<int64_t, int32_t>> all;
  for (int p = 0; p < parts; ++p) {
    mi = std::max(mi, max_in[static_cast<size_t>(p)]);
    all.insert(all.end(), tops[static_cast<size_t>(p)].begin(), tops[static_cast<size_t>(p)].end());
  }
  g->sigma_limit = ~0ull / static_cast<unsigned long long>(mi + 1);
  std::sort(all.begin(), all.end());
  g->landmarks.clear();
  for (size_t i = 0; i < all.size() && i < static_cast<size_t>(kLandmarks); ++i)
    g->landmarks.push_back(all[i].second);
}

int finish_handle(lgbc_graph* g, const int64_t* rowptr, const int64_t* in_rowptr,
                  const int32_t* colidx, const int32_t* in_colidx) {
  degree_pass(g, rowptr, in_rowptr);
  const int directed = g->directed;
  return build_hubs(g, rowptr, colidx, directed ? in_rowptr : rowptr, directed ? in_colidx : colidx,
                    g->tune.hub_degree, g->tune.hub_order);
}

}  // namespace lgbc::api

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

namespace lgbc::api {

// Level-synchronous BFS over dg from d_src[0, nsrc) into d_dist, which the
// caller has filled (kUnreached, and any other value on vertices the search
// must treat as already visited).
int run_bfs(lgbc_graph* g, const DevGraph& dg, int64_t nsrc) {
  BfsBuffers b{g->bfs.queue, {g->bfs.bm0, g->bfs.bm1}, g->bfs.ctl, g->bfs.large};
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

}  // namespace lgbc::api

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
  if (!(t->alpha > 0) || !(t->beta > 0) || t->lanes < 1 || t->lanes > kWideLanes ||
      t->hub_degree < 1 || t->dense_edges < 0 || t->segment_degree < 0 ||
      (t->source_order != 0 && t->source_order != 1) || (t->graph_loop != 0 && t->graph_loop != 1) ||
      t->stack_vertices < 0 || t->hub_order < 0 || t->hub_order > 2 ||
      (t->dependency_df32 != 0 && t->dependency_df32 != 1))
    return fail(LGBC_EINVAL,
                "tuning out of range (alpha, beta > 0; 1 <= lanes <= 128; hub_degree >= 1; "
                "dense_edges, segment_degree, stack_vertices >= 0; hub_order 0..2; "
                "dependency_df32 0 or 1)");
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
