// api_learned.cu -- entry points of the learned source proposal (features, core
// numbers, dependency mass, distance statistics, weighted Brandes, proposal).
#include "api_internal.h"

using namespace lgbc;
using namespace lgbc::api;

// ---------------------------------------------------------------------------
// Learned source proposal (learned.cu, mlp.cu)
// ---------------------------------------------------------------------------
namespace lgbc::api {

int ensure_learned(lgbc_graph* g) {
  LearnedWorkspace& w = g->learned;
  if (w.core) return LGBC_OK;
  const size_t n = static_cast<size_t>(g->n);
  const size_t tiles = static_cast<size_t>(proposal_tiles(g->n));
  LGBC_TRY(dev_alloc(&w.core, n));
  LGBC_TRY(dev_alloc(&w.flag, n));
  LGBC_TRY(dev_alloc(&w.list, n));
  LGBC_TRY(dev_alloc(&w.large, n));
  LGBC_TRY(dev_alloc(&w.log_v, n));
  LGBC_TRY(dev_alloc(&w.log_old, n));
  LGBC_TRY(dev_alloc(&w.hub_v, n));
  LGBC_TRY(dev_alloc(&w.hub_old, n));
  LGBC_TRY(dev_alloc(&w.counters, 5));
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
  LGBC_CUDA(cudaMemsetAsync(w.counters, 0, 5 * 8, g->stream));
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
    const CorePassBuffers cb{w.counters + 1, w.counters + 4, w.counters + 3, w.log_v,
                             w.log_old,      w.hub_v,        w.hub_old,      w.large};
    g->launches += core_pass(g->cfg, g->stream, dg, list, nlist, w.core, w.flag, cb);
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

}  // namespace lgbc::api

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

