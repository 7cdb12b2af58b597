// api_more.cu -- the autotuner, stress centrality, BFS parents / has_path and
// graph ingest on the device.
#include "api_internal.h"

using namespace lgbc;
using namespace lgbc::api;

// ---------------------------------------------------------------------------
// Autotuner
// ---------------------------------------------------------------------------
namespace lgbc::api {

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
    if (std::sscanf(line, "%255s %lf %lf %d %d %d %d %d %d %d %d", key, &t.alpha, &t.beta,
                    &t.hub_degree, &t.lanes, &t.dense_edges, &t.segment_degree, &t.source_order,
                    &t.graph_loop, &t.stack_vertices, &t.hub_order) == 11 &&
        sig == key && t.alpha > 0 && t.beta > 0 && t.lanes >= 1 && t.lanes <= kWideLanes &&
        t.hub_degree >= 1 && t.dense_edges >= 0 && t.segment_degree >= 0 &&
        (t.source_order == 0 || t.source_order == 1) && (t.graph_loop == 0 || t.graph_loop == 1) &&
        t.stack_vertices >= 0 && t.hub_order >= 0 && t.hub_order <= 2) {
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

}  // namespace lgbc::api

extern "C" int lgbc_tune(lgbc_graph* g, const char* cache_path) {
  LGBC_TRY(check_graph(g));
  std::lock_guard<std::mutex> lock(g->mu);
  LGBC_TRY(use_device(g));
  reset_stats(g);
  const std::string sig = tune_signature(g);
  lgbc_tuning cached{};
  if (tune_from_cache(cache_path, sig, &cached)) {
    cached.dependency_df32 = g->tune.dependency_df32;  // a precision choice, not tuned
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
    const int lanes[] = {32, 48, 64, 128};
    const double alphas[] = {2.0, 4.0, 8.0, 14.0, 24.0, 48.0};
    const double betas[] = {6.0, 12.0, 24.0, 48.0, 96.0};
    const int dense[] = {4, 8, 16, 32};
    const int segs[] = {0, 1 << 30};
    const int orders[] = {0, 1, 2};
    LGBC_TRY(try_field([](lgbc_tuning& c, int v) { c.hub_degree = v; }, hubs));
    LGBC_TRY(try_field([](lgbc_tuning& c, int v) { c.lanes = v; }, lanes));
    LGBC_TRY(try_field([](lgbc_tuning& c, double v) { c.alpha = v; }, alphas));
    LGBC_TRY(try_field([](lgbc_tuning& c, double v) { c.beta = v; }, betas));
    LGBC_TRY(try_field([](lgbc_tuning& c, int v) { c.dense_edges = v; }, dense));
    LGBC_TRY(try_field([](lgbc_tuning& c, int v) { c.segment_degree = v; }, segs));
    LGBC_TRY(try_field([](lgbc_tuning& c, int v) { c.hub_order = v; }, orders));
  }
  g->tune = best;
  LGBC_TRY(ensure_hubs(g));
  if (cache_path) {
    FILE* f = std::fopen(cache_path, "a");
    if (!f) return fail(LGBC_EINVAL, std::string("cannot append to tuning cache ") + cache_path);
    std::fprintf(f, "%s %.17g %.17g %d %d %d %d %d %d %d %d\n", sig.c_str(), best.alpha, best.beta,
                 best.hub_degree, best.lanes, best.dense_edges, best.segment_degree,
                 best.source_order, best.graph_loop, best.stack_vertices, best.hub_order);
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
// Path counts (DijkstraState.pathcounts / .dists with unit weights)
// ---------------------------------------------------------------------------
extern "C" int lgbc_path_counts(lgbc_graph* g, const int32_t* src, int64_t nsrc,
                                double* sigma_out, int32_t* dist_out) {
  LGBC_TRY(check_graph(g));
  std::lock_guard<std::mutex> lock(g->mu);
  LGBC_TRY(use_device(g));
  LGBC_TRY(check_sources(g, src, nsrc));
  if (nsrc > 0 && g->n > 0 && !sigma_out) return fail(LGBC_EINVAL, "null output");
  reset_stats(g);
  if (nsrc == 0 || g->n == 0) return LGBC_OK;
  LGBC_TRY(ensure_ms(g, true));
  LGBC_TRY(ensure_src(g, nsrc));
  LGBC_CUDA(cudaMemcpyAsync(g->d_src, src, static_cast<size_t>(nsrc) * 4, cudaMemcpyHostToDevice,
                            g->stream));
  const int64_t n = g->n;
  const int lanes = kMaxLanes;  // one-word batches
  double* d_pc = nullptr;
  int32_t* d_d = nullptr;
  LGBC_TRY(dev_alloc(&d_pc, static_cast<size_t>(lanes) * static_cast<size_t>(n)));
  std::unique_ptr<double, void (*)(double*)> g1(d_pc, [](double* q) { cudaFree(q); });
  LGBC_TRY(dev_alloc(&d_d, static_cast<size_t>(lanes) * static_cast<size_t>(n)));
  std::unique_ptr<int32_t, void (*)(int32_t*)> g2(d_d, [](int32_t* q) { cudaFree(q); });
  for (int64_t s0 = 0; s0 < nsrc; s0 += lanes) {
    const int nl = static_cast<int>(std::min<int64_t>(lanes, nsrc - s0));
    const int64_t cells = static_cast<int64_t>(nl) * n;
    PathExport px;
    px.sigma = d_pc;
    px.dist = d_d;
    px.ld = n;
    int rc = LGBC_OK;
    for (int kind : {static_cast<int>(kSigmaU64), static_cast<int>(kSigmaF64)}) {
      // unreached: pathcounts 0 and distance typemax, as dijkstra.jl:66-69 start them
      g->launches += fill_f64(g->cfg, g->stream, d_pc, cells, 0.0);
      g->launches += fill_i32(g->cfg, g->stream, d_d, cells, kUnreached);
      rc = run_ms_batch(g, g->d_src + s0, nl, kind, nullptr, nullptr, 0, Seeds(), nullptr,
                        nullptr, nullptr, &px);
      if (rc != 1) break;  // 1: a count may pass 2^64, replay with FP64 counts
      g->stats.wide_batches++;
    }
    if (rc != LGBC_OK) return rc < 0 ? rc : fail(LGBC_ECUDA, "internal: FP64 replay overflowed");
    LGBC_CUDA(cudaMemcpyAsync(sigma_out + s0 * n, d_pc, static_cast<size_t>(cells) * 8,
                              cudaMemcpyDeviceToHost, g->stream));
    if (dist_out)
      LGBC_CUDA(cudaMemcpyAsync(dist_out + s0 * n, d_d, static_cast<size_t>(cells) * 4,
                                cudaMemcpyDeviceToHost, g->stream));
    g->stats.batches++;
  }
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
namespace lgbc::api {

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

}  // namespace lgbc::api

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

