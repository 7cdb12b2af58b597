// api_many.cu -- lgbc_betweenness_many: exact betweenness of many graphs as
// disjoint unions of similar-size graphs.
#include <atomic>

#include "api_internal.h"

using namespace lgbc;
using namespace lgbc::api;

// ---------------------------------------------------------------------------
// Exact betweenness of many graphs (disjoint unions, one lane per source
// index in every graph of a group).
// ---------------------------------------------------------------------------
namespace lgbc::api {

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
  std::vector<int32_t> sv;
  std::vector<uint64_t> sm;
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
      sm.push_back(1ull << j);
    }
  }
  if (sv.empty()) return LGBC_OK;
  const int64_t N = g->n;
  LGBC_TRY(ensure_ms(g, false));
  int32_t* d_dist = nullptr;  // nl x N distances | seed vertices
  LGBC_TRY(dev_alloc(&d_dist, static_cast<size_t>(nl) * static_cast<size_t>(N) + sv.size()));
  std::unique_ptr<int32_t, cudaError_t (*)(void*)> guard(d_dist, cudaFree);
  uint64_t* d_sm = nullptr;
  LGBC_TRY(dev_alloc(&d_sm, sm.size()));
  std::unique_ptr<uint64_t, cudaError_t (*)(void*)> guard2(d_sm, cudaFree);
  int32_t* d_sv = d_dist + static_cast<int64_t>(nl) * N;
  LGBC_CUDA(cudaMemcpyAsync(d_sv, sv.data(), sv.size() * 4, cudaMemcpyHostToDevice, g->stream));
  LGBC_CUDA(cudaMemcpyAsync(d_sm, sm.data(), sm.size() * 8, cudaMemcpyHostToDevice, g->stream));
  g->launches += fill_i32(g->cfg, g->stream, d_dist, static_cast<int64_t>(nl) * N, kUnreached);
  Seeds sd;
  sd.v = d_sv;
  sd.mask = d_sm;
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
  std::vector<int32_t> sv, act_src;
  std::vector<uint64_t> sm;
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
  // L lanes per batch (the handle's default batch width), W lane words
  const int L = std::max(1, std::min<int>(kWideLanes, g->tune.lanes));
  const int W = lane_words(L);
  if (g->tune.source_order == 1 && maxa > L)
    LGBC_TRY(order_many(g, grp, voff, act));
  // batch b, lane l holds the (L b + l)-th ordered source of every graph;
  // W mask words per seed and per (batch, graph) mark
  const int64_t nb = (maxa + L - 1) / L;
  const LaneSet all = lane_set(L, W);
  std::vector<int64_t> bstart(static_cast<size_t>(nb + 1), 0);
  std::vector<uint64_t> marks(static_cast<size_t>(nb) * grp.size() * W);
  for (int64_t b = 0; b < nb; ++b) {
    for (size_t k = 0; k < grp.size(); ++k) {
      LaneSet seeded{};
      for (int l = 0; l < L; ++l) {
        const int64_t i = b * L + l;
        if (i < static_cast<int64_t>(act[k].size())) {
          sv.push_back(static_cast<int32_t>(voff[k] + act[k][static_cast<size_t>(i)]));
          for (int q = 0; q < W; ++q) sm.push_back(q == (l >> 6) ? 1ull << (l & 63) : 0ull);
          seeded.w[l >> 6] |= 1ull << (l & 63);
        }
      }
      for (int q = 0; q < W; ++q)
        marks[(static_cast<size_t>(b) * grp.size() + k) * W + q] = all.w[q] & ~seeded.w[q];
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
  uint64_t* d_sm = nullptr;
  LGBC_TRY(dev_alloc(&d_sv, sv.size()));
  std::unique_ptr<int32_t, cudaError_t (*)(void*)> g1(d_sv, cudaFree);
  LGBC_TRY(dev_alloc(&d_sm, sm.size()));
  std::unique_ptr<uint64_t, cudaError_t (*)(void*)> g2(d_sm, cudaFree);
  if (!sv.empty()) {
    LGBC_CUDA(cudaMemcpyAsync(d_sv, sv.data(), sv.size() * 4, cudaMemcpyHostToDevice, g->stream));
    LGBC_CUDA(cudaMemcpyAsync(d_sm, sm.data(), sm.size() * 8, cudaMemcpyHostToDevice, g->stream));
  }
  if (!g->d_bc) LGBC_TRY(dev_alloc(&g->d_bc, static_cast<size_t>(N)));
  g->launches += fill_f64(g->cfg, g->stream, g->d_bc, N, 0.0);
  if (!sv.empty()) LGBC_TRY(ensure_ms(g, true, W));
  for (int64_t b = 0; b < nb; ++b) {
    Seeds sd;
    sd.v = d_sv + bstart[static_cast<size_t>(b)];
    sd.mask = d_sm + bstart[static_cast<size_t>(b)] * W;
    sd.count = bstart[static_cast<size_t>(b + 1)] - bstart[static_cast<size_t>(b)];
    if (sd.count == 0) continue;
    sd.seg_off = d_voff;
    sd.seg_mark = d_marks + static_cast<size_t>(b) * grp.size() * W;
    sd.nseg = static_cast<int64_t>(grp.size());
    int rc = run_ms_batch(g, nullptr, L, dep_kind(g), g->d_bc, nullptr, 0, sd);
    if (rc == 1) rc = run_ms_batch(g, nullptr, L, kSigmaF64, g->d_bc, nullptr, 0, sd);
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

// Runs the groups kManyInFlight at a time: each group has its own union
// handle and stream, so while one group's batches run on the GPU the next
// group's host work (union CSR, handle set-up, source ordering, seeds) goes
// on in another host thread, and the groups' latency-bound kernels overlap
// on the GPU (1,024 BA graphs on GB300: 12.08 s one at a time, 9.65 s two,
// 8.79 s three).  Groups write disjoint ranges of bc_raw_out.
// The first failure stops the remaining groups; its code and message are
// returned in the calling thread.
int run_groups(const std::vector<std::vector<ManyGraph>>& groups, int endpoints,
               double* bc_raw_out) {
  constexpr size_t kManyInFlight = 3;
  int dev = 0;
  LGBC_CUDA(cudaGetDevice(&dev));
  std::atomic<size_t> next{0};
  std::mutex mu;
  int first_rc = LGBC_OK;
  std::string first_msg;
  auto record = [&](int rc, const std::string& msg) {
    std::lock_guard<std::mutex> lock(mu);
    if (first_rc == LGBC_OK) {
      first_rc = rc;
      first_msg = msg;
    }
  };
  auto stopped = [&]() {
    std::lock_guard<std::mutex> lock(mu);
    return first_rc != LGBC_OK;
  };
  auto worker = [&]() {
    const cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) {
      record(LGBC_ECUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
      return;
    }
    for (size_t i = next.fetch_add(1); i < groups.size() && !stopped(); i = next.fetch_add(1)) {
      int rc;
      try {
        rc = many_group(groups[i], endpoints, bc_raw_out);
      } catch (const std::bad_alloc&) {
        rc = fail(LGBC_ENOMEM, "host allocation failed");
      } catch (const std::exception& ex) {  // never let one leave a worker thread
        rc = fail(LGBC_EINVAL, std::string("many-graph union: ") + ex.what());
      }
      if (rc != LGBC_OK) {
        record(rc, g_last_error);
        return;
      }
    }
  };
  std::vector<std::thread> extra;
  for (size_t t = 1; t < std::min(kManyInFlight, groups.size()); ++t) extra.emplace_back(worker);
  worker();
  for (auto& t : extra) t.join();
  if (first_rc != LGBC_OK) return fail(first_rc, first_msg);
  return LGBC_OK;
}

}  // namespace lgbc::api

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
  std::vector<std::vector<ManyGraph>> groups(1);
  int64_t gv = 0;
  for (size_t oi = 0; oi < order.size(); ++oi) {
    const ManyGraph& m = gs[order[oi]];
    if (!groups.back().empty() && gv + m.n > kGroupVertices) {
      groups.emplace_back();
      gv = 0;
    }
    groups.back().push_back(m);
    gv += m.n;
  }
  return run_groups(groups, endpoints, bc_raw_out);
}
