// lg_oracle.cpp -- CPU oracle for the GB300 betweenness-centrality / BFS path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in plain C++17, the reference
// algorithms of LightGraphs.jl v1.3.5 that the CUDA library replaces.  It is
// the checker for the GPU results and the timed CPU baseline; nothing in the
// product library links or calls it.  Only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline / reference arm load it.
//
// Every function cites the reference file:line it follows (paths relative to
// the LightGraphs.jl project root).  Graphs arrive as 0-based CSR:
// rowptr[n+1] (int64), colidx[nnz] (int32), each row sorted ascending --
// exactly the flattening of SimpleGraph.fadjlist / SimpleDiGraph.fadjlist
// (src/SimpleGraphs/simplegraph.jl:8-16, simpledigraph.jl:8-21).  For a
// digraph the in-CSR (badjlist) is passed too.
//
// Parity status: pinned.  tests/test_oracle_golden.py checks this oracle
// against the reference's golden vector test/testdata/graph-50-500-bc.txt
// (Float32-equal, test/centrality/betweenness.jl:8-13), the endpoints triple
// (:15-17), the self-loop / 2-vertex / path cases (:28-41), the doc examples
// (src/centrality/betweenness.jl:32-43), the Dijkstra sigma / predecessor /
// closest-vertex fixtures (test/shortestpaths/dijkstra.jl:70-99) and the
// gdistances fixtures (test/traversals/bfs.jl:29-35).

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

constexpr int32_t kUnreached32 = std::numeric_limits<int32_t>::max();
constexpr int64_t kUnreached64 = std::numeric_limits<int64_t>::max();

struct Csr {
  int64_t n;
  const int64_t* rowptr;
  const int32_t* colidx;
  int64_t deg(int64_t v) const { return rowptr[v + 1] - rowptr[v]; }
};

// Indexed binary min-heap keyed by distance, standing in for
// DataStructures.PriorityQueue{U,T} (src/shortestpaths/dijkstra.jl:73).  Only
// the tie order among equal keys can differ from the reference's heap, and
// with unit weights that changes summation order, never values.
class IndexedHeap {
 public:
  explicit IndexedHeap(int64_t n) : pos_(n, -1) {}
  bool empty() const { return v_.empty(); }
  // H[v] = key (insert or update), dijkstra.jl:80,107,115
  void set(int32_t v, int64_t key) {
    int64_t i = pos_[v];
    if (i < 0) {
      v_.push_back(v);
      k_.push_back(key);
      i = static_cast<int64_t>(v_.size()) - 1;
      pos_[v] = i;
      up(i);
    } else {
      int64_t old = k_[i];
      k_[i] = key;
      if (key < old) up(i); else down(i);
    }
  }
  // dequeue!(H), dijkstra.jl:87
  int32_t pop() {
    int32_t top = v_[0];
    pos_[top] = -1;
    int64_t last = static_cast<int64_t>(v_.size()) - 1;
    if (last > 0) {
      v_[0] = v_[last];
      k_[0] = k_[last];
      pos_[v_[0]] = 0;
    }
    v_.pop_back();
    k_.pop_back();
    if (!v_.empty()) down(0);
    return top;
  }

 private:
  void swap_at(int64_t a, int64_t b) {
    std::swap(v_[a], v_[b]);
    std::swap(k_[a], k_[b]);
    pos_[v_[a]] = a;
    pos_[v_[b]] = b;
  }
  void up(int64_t i) {
    while (i > 0) {
      int64_t p = (i - 1) / 2;
      if (k_[i] < k_[p]) { swap_at(i, p); i = p; } else break;
    }
  }
  void down(int64_t i) {
    int64_t m = static_cast<int64_t>(v_.size());
    for (;;) {
      int64_t l = 2 * i + 1, r = l + 1, s = i;
      if (l < m && k_[l] < k_[s]) s = l;
      if (r < m && k_[r] < k_[s]) s = r;
      if (s == i) break;
      swap_at(i, s);
      i = s;
    }
  }
  std::vector<int32_t> v_;
  std::vector<int64_t> k_;
  std::vector<int64_t> pos_;
};

// DijkstraState (src/shortestpaths/dijkstra.jl:6-12) with unit weights.
struct DijkstraState {
  std::vector<int64_t> dists;
  std::vector<double> pathcounts;
  std::vector<std::vector<int32_t>> preds;
  std::vector<int32_t> closest;
};

// dijkstra_shortest_paths(g, s, DefaultDistance; allpaths=true,
// trackvertices=true), src/shortestpaths/dijkstra.jl:59-141, single source
// (:143-144).  DefaultDistance has every entry 1 (src/distance.jl:8-21).
void dijkstra_allpaths(const Csr& g, int32_t src, DijkstraState& st) {
  const int64_t n = g.n;
  st.dists.assign(n, kUnreached64);               // :65
  std::vector<char> visited(n, 0);                // :67
  st.pathcounts.assign(n, 0.0);                   // :69
  st.preds.assign(n, std::vector<int32_t>());     // :70 (one array per vertex)
  st.closest.clear();
  st.closest.reserve(n);                          // :83-84
  IndexedHeap H(n);                               // :71
  st.dists[src] = 0;                              // :75-80
  visited[src] = 1;
  st.pathcounts[src] = 1.0;
  H.set(src, 0);
  while (!H.empty()) {                            // :86
    int32_t u = H.pop();
    st.closest.push_back(u);                      // :89-91
    int64_t d = st.dists[u];
    for (int64_t e = g.rowptr[u]; e < g.rowptr[u + 1]; ++e) {
      int32_t v = g.colidx[e];
      int64_t alt = d + 1;                        // :95
      if (!visited[v]) {                          // :97-106
        visited[v] = 1;
        st.dists[v] = alt;
        st.pathcounts[v] += st.pathcounts[u];
        st.preds[v].assign(1, u);
        H.set(v, alt);
      } else if (alt < st.dists[v]) {             // :108-116 (never taken
        st.dists[v] = alt;                        //  with unit weights;
        st.pathcounts[v] = st.pathcounts[u];      //  kept for fidelity)
        st.preds[v].assign(1, u);
        H.set(v, alt);
      } else if (alt == st.dists[v]) {            // :117-122
        st.pathcounts[v] += st.pathcounts[u];
        st.preds[v].push_back(u);
      }
    }
  }
  for (int64_t s = 0; s < n; ++s)                 // :126-132 unreached
    if (!visited[s]) st.closest.push_back(static_cast<int32_t>(s));
  st.pathcounts[src] = 1.0;                       // :134-138
  st.preds[src].clear();
}

// _accumulate_basic! / _accumulate_endpoints!
// (src/centrality/betweenness.jl:81-107, :109-134) on a DijkstraState.
void accumulate_faithful(const DijkstraState& st, int32_t s, int endpoints,
                         std::vector<double>& delta, double* bc) {
  const int64_t n = static_cast<int64_t>(st.pathcounts.size());
  delta.assign(n, 0.0);
  if (endpoints) bc[s] += static_cast<double>(st.closest.size()) - 1.0;  // :122
  for (auto it = st.closest.rbegin(); it != st.closest.rend(); ++it) {
    int32_t w = *it;
    double coeff = (1.0 + delta[w]) / st.pathcounts[w];                  // :96,125
    for (int32_t v : st.preds[w]) delta[v] += st.pathcounts[v] * coeff;  // :97-101
    if (w != s) bc[w] += endpoints ? (delta[w] + 1.0) : delta[w];       // :102-104
  }
}

// The same accumulation over a BFS order: sigma and the predecessor relation
// are identical to the unit-weight Dijkstra state above (predecessors of w are
// the in-neighbours v with d[v] == d[w] - 1), only the visiting order among
// equal distances -- and therefore the floating-point summation order --
// differs.  This is the "fast" CPU restatement.
struct BfsWork {
  std::vector<int32_t> dist, order;
  std::vector<double> sigma, delta;
};

void brandes_bfs(const Csr& out, const Csr& in, int32_t s, int endpoints,
                 BfsWork& w, double* bc) {
  const int64_t n = out.n;
  w.dist.assign(n, -1);
  w.sigma.assign(n, 0.0);
  w.delta.assign(n, 0.0);
  w.order.clear();
  w.order.reserve(n);
  w.dist[s] = 0;
  w.sigma[s] = 1.0;
  w.order.push_back(s);
  for (size_t head = 0; head < w.order.size(); ++head) {
    int32_t u = w.order[head];
    int32_t du = w.dist[u];
    for (int64_t e = out.rowptr[u]; e < out.rowptr[u + 1]; ++e) {
      int32_t v = out.colidx[e];
      if (w.dist[v] < 0) {
        w.dist[v] = du + 1;
        w.order.push_back(v);
      }
      if (w.dist[v] == du + 1) w.sigma[v] += w.sigma[u];
    }
  }
  const int64_t reached = static_cast<int64_t>(w.order.size());
  if (endpoints) bc[s] += static_cast<double>(n) - 1.0;   // |S| is always n
  for (int64_t i = reached - 1; i >= 0; --i) {
    int32_t x = w.order[i];
    double coeff = (1.0 + w.delta[x]) / w.sigma[x];
    int32_t dx = w.dist[x];
    if (dx > 0) {
      for (int64_t e = in.rowptr[x]; e < in.rowptr[x + 1]; ++e) {
        int32_t v = in.colidx[e];
        if (w.dist[v] == dx - 1) w.delta[v] += w.sigma[v] * coeff;
      }
    }
    if (x != s) bc[x] += endpoints ? (w.delta[x] + 1.0) : w.delta[x];
  }
  if (endpoints) {
    // unreached vertices still receive delta[w] + 1 = 1 (betweenness.jl:126-131
    // walks all n vertices because dijkstra.jl:126-132 pads closest_vertices).
    for (int64_t v = 0; v < n; ++v)
      if (w.dist[v] < 0) bc[v] += 1.0;
  }
}

// degree(g, v): in+out for digraphs, length(fadjlist[v]) for graphs
// (src/core.jl:66-67).
inline int64_t degree_of(const Csr& out, const Csr* in, int directed, int64_t v) {
  return out.deg(v) + (directed ? in->deg(v) : 0);
}

// Runs `fn(source_index, thread_id)` over [0, nsrc) on `nthreads` threads with
// dynamic claiming, the shape of Parallel.threaded_betweenness_centrality's
// @threads loop (src/Parallel/centrality/betweenness.jl:55-61).
template <class Fn>
void parallel_over(int64_t nsrc, int nthreads, Fn fn) {
  if (nthreads <= 1 || nsrc <= 1) {
    for (int64_t i = 0; i < nsrc; ++i) fn(i, 0);
    return;
  }
  std::atomic<int64_t> next(0);
  std::vector<std::thread> pool;
  for (int t = 0; t < nthreads; ++t) {
    pool.emplace_back([&, t]() {
      for (;;) {
        int64_t i = next.fetch_add(1);
        if (i >= nsrc) break;
        fn(i, t);
      }
    });
  }
  for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

// gdistances!(g, source, vert_level) -- src/traversals/bfs.jl:95-124; the
// level-synchronous BFS with a visited bit vector and a sorted level queue
// (:121).  Multi-source: every source gets level 0 (:103-107).  Unreached
// vertices keep INT32_MAX (the caller maps it to typemax(T), :141).
int orc_gdistances(int64_t n, const int64_t* rowptr, const int32_t* colidx,
                   const int32_t* src, int64_t nsrc, int32_t* dist) {
  for (int64_t i = 0; i < nsrc; ++i)
    if (src[i] < 0 || src[i] >= n) return -1;
  std::fill(dist, dist + n, kUnreached32);
  std::vector<char> visited(n, 0);
  std::vector<int32_t> cur, next;
  cur.reserve(n);
  next.reserve(n);
  int32_t n_level = 1;
  for (int64_t i = 0; i < nsrc; ++i) {
    dist[src[i]] = 0;
    visited[src[i]] = 1;
    cur.push_back(src[i]);
  }
  while (!cur.empty()) {
    for (int32_t v : cur) {
      for (int64_t e = rowptr[v]; e < rowptr[v + 1]; ++e) {
        int32_t i = colidx[e];
        if (!visited[i]) {
          next.push_back(i);
          dist[i] = n_level;
          visited[i] = 1;
        }
      }
    }
    ++n_level;
    cur.clear();
    std::swap(cur, next);
    std::sort(cur.begin(), cur.end());
  }
  return 0;
}

// nsrc independent single-source gdistances (the loop above per source), one
// source per host thread: dist[i * n + v] is the level of v from src[i].
int orc_gdistances_many(int64_t n, const int64_t* rowptr, const int32_t* colidx,
                        const int32_t* src, int64_t nsrc, int nthreads, int32_t* dist) {
  for (int64_t i = 0; i < nsrc; ++i)
    if (src[i] < 0 || src[i] >= n) return -1;
  parallel_over(nsrc, nthreads, [&](int64_t i, int) {
    orc_gdistances(n, rowptr, colidx, src + i, 1, dist + i * n);
  });
  return 0;
}

// dijkstra_shortest_paths(g, s; allpaths=true, trackvertices=true) with unit
// weights (src/shortestpaths/dijkstra.jl:59-144).  Outputs: dists (INT64_MAX
// = unreached), pathcounts, closest_vertices (n entries), predecessors as a
// CSR (pred_off[n+1], pred[...]) in push order.  Returns the number of
// predecessor entries, or -1 if pred_cap is too small / bad source.
int64_t orc_dijkstra(int64_t n, const int64_t* rowptr, const int32_t* colidx,
                     int32_t s, int64_t* dists, double* pathcounts,
                     int32_t* closest, int64_t* pred_off, int32_t* pred,
                     int64_t pred_cap) {
  if (s < 0 || s >= n) return -1;
  Csr g{n, rowptr, colidx};
  DijkstraState st;
  dijkstra_allpaths(g, s, st);
  int64_t total = 0;
  for (int64_t v = 0; v < n; ++v) total += static_cast<int64_t>(st.preds[v].size());
  if (total > pred_cap) return -1;
  int64_t o = 0;
  for (int64_t v = 0; v < n; ++v) {
    dists[v] = st.dists[v];
    pathcounts[v] = st.pathcounts[v];
    closest[v] = st.closest[v];
    pred_off[v] = o;
    for (int32_t u : st.preds[v]) pred[o++] = u;
  }
  pred_off[n] = o;
  return total;
}

// Unscaled betweenness over an explicit source list:
// src/centrality/betweenness.jl:46-75 without the final _rescale! (:69-73),
// or equally Parallel.threaded_betweenness_centrality
// (src/Parallel/centrality/betweenness.jl:42-72) before its rescale.
// Sources with degree(g, s) == 0 are skipped (:58, Parallel :53).
// mode 0 = faithful (heap Dijkstra + per-vertex predecessor vectors, the
// reference's own cost model); mode 1 = BFS Brandes (same values).
// Per-thread FP64 buffers are reduced in thread order (Parallel :52,63).
int orc_betweenness(int64_t n, const int64_t* rowptr, const int32_t* colidx,
                    const int64_t* in_rowptr, const int32_t* in_colidx,
                    int directed, const int32_t* src, int64_t nsrc,
                    int endpoints, int mode, int nthreads, double* bc_raw) {
  for (int64_t i = 0; i < nsrc; ++i)
    if (src[i] < 0 || src[i] >= n) return -1;
  if (directed && (!in_rowptr || !in_colidx)) return -1;
  Csr out{n, rowptr, colidx};
  Csr in = directed ? Csr{n, in_rowptr, in_colidx} : out;
  if (nthreads < 1) nthreads = 1;
  std::vector<std::vector<double>> local(nthreads, std::vector<double>(n, 0.0));
  // vs_active = findall(x -> degree(g, x) > 0, vs)
  std::vector<int32_t> active;
  active.reserve(nsrc);
  for (int64_t i = 0; i < nsrc; ++i)
    if (degree_of(out, &in, directed, src[i]) > 0) active.push_back(src[i]);
  const int64_t na = static_cast<int64_t>(active.size());
  if (mode == 0) {
    std::vector<DijkstraState> st(nthreads);
    std::vector<std::vector<double>> delta(nthreads);
    parallel_over(na, nthreads, [&](int64_t i, int t) {
      dijkstra_allpaths(out, active[i], st[t]);
      accumulate_faithful(st[t], active[i], endpoints, delta[t], local[t].data());
    });
  } else {
    std::vector<BfsWork> work(nthreads);
    parallel_over(na, nthreads, [&](int64_t i, int t) {
      brandes_bfs(out, in, active[i], endpoints, work[t], local[t].data());
    });
  }
  std::fill(bc_raw, bc_raw + n, 0.0);
  for (int t = 0; t < nthreads; ++t)
    for (int64_t v = 0; v < n; ++v) bc_raw[v] += local[t][v];
  return 0;
}

// _rescale!(betweenness, n, normalize, directed, k),
// src/centrality/betweenness.jl:136-160.  (n - 1) * (n - 2) is evaluated in
// Int64: Julia promotes nv(g)::T with the Int64 literals 1 and 2, so no
// narrower eltype can overflow there.
void orc_rescale(double* bc, int64_t n, int normalize, int directed, int64_t k) {
  bool do_scale;
  double scale = 1.0;
  if (normalize) {
    if (n <= 2) {
      do_scale = false;
    } else {
      do_scale = true;
      scale = 1.0 / static_cast<double>((n - 1) * (n - 2));
    }
  } else {
    if (!directed) { do_scale = true; scale = 1.0 / 2.0; }
    else do_scale = false;
  }
  if (do_scale) {
    if (k > 0) scale = scale * static_cast<double>(n) / static_cast<double>(k);
    for (int64_t v = 0; v < n; ++v) bc[v] *= scale;
  }
}

// Per-source dependency mass sum_{v != s} delta_s(v) (the total that
// _accumulate_basic!, src/centrality/betweenness.jl:81-107, adds to the
// betweenness vector for source s; 0 for sources of degree 0, :58), and the
// weighted accumulation sum_i w_i * delta_{s_i}(v) used by importance-sampled
// estimators.  Either output may be NULL.
int orc_dependency(int64_t n, const int64_t* rowptr, const int32_t* colidx,
                   const int64_t* in_rowptr, const int32_t* in_colidx, int directed,
                   const int32_t* src, const double* w, int64_t nsrc, double* mass_out,
                   double* bc_weighted_out) {
  for (int64_t i = 0; i < nsrc; ++i)
    if (src[i] < 0 || src[i] >= n) return -1;
  if (directed && (!in_rowptr || !in_colidx)) return -1;
  Csr out{n, rowptr, colidx};
  Csr in = directed ? Csr{n, in_rowptr, in_colidx} : out;
  BfsWork wk;
  std::vector<double> tmp(n, 0.0);
  if (bc_weighted_out) std::fill(bc_weighted_out, bc_weighted_out + n, 0.0);
  for (int64_t i = 0; i < nsrc; ++i) {
    const int32_t s = src[i];
    double mass = 0.0;
    if (degree_of(out, &in, directed, s) > 0) {
      std::fill(tmp.begin(), tmp.end(), 0.0);
      brandes_bfs(out, in, s, 0, wk, tmp.data());
      for (int64_t v = 0; v < n; ++v) {
        mass += tmp[v];
        if (bc_weighted_out) bc_weighted_out[v] += (w ? w[i] : 1.0) * tmp[v];
      }
    }
    if (mass_out) mass_out[i] = mass;
  }
  return 0;
}

// stress_centrality(g, vs) (src/centrality/stress.jl:33-49) with
// _stress_accumulate_basic! (:51-77) on the Dijkstra state of every source of
// degree > 0.  Julia's Int64 arithmetic wraps; uint64 arithmetic wraps
// identically (two's complement), so the sums are kept in uint64.
int orc_stress(int64_t n, const int64_t* rowptr, const int32_t* colidx,
               const int64_t* in_rowptr, const int32_t* in_colidx, int directed,
               const int32_t* src, int64_t nsrc, int64_t* stress_out) {
  for (int64_t i = 0; i < nsrc; ++i)
    if (src[i] < 0 || src[i] >= n) return -1;
  if (directed && (!in_rowptr || !in_colidx)) return -1;
  Csr out{n, rowptr, colidx};
  Csr in = directed ? Csr{n, in_rowptr, in_colidx} : out;
  std::vector<uint64_t> stress(n, 0);
  std::vector<uint64_t> delta(n);
  DijkstraState st;
  for (int64_t i = 0; i < nsrc; ++i) {
    const int32_t s = src[i];
    if (degree_of(out, &in, directed, s) == 0) continue;        // :38
    dijkstra_allpaths(out, s, st);                               // :39
    std::fill(delta.begin(), delta.end(), 0);                    // :57
    st.preds[s].clear();                                         // :62
    for (auto it = st.closest.rbegin(); it != st.closest.rend(); ++it) {  // :64-65
      const int32_t w = *it;
      for (int32_t v : st.preds[w]) delta[v] += delta[w] + 1;    // :66-70
      delta[w] *= static_cast<uint64_t>(st.preds[w].size());     // :72
      if (w != s) stress[w] += delta[w];                         // :73-75
    }
  }
  for (int64_t v = 0; v < n; ++v) stress_out[v] = static_cast<int64_t>(stress[v]);
  return 0;
}

// core_number(g) for a graph without self-loops: the bin-sort cores
// decomposition of Batagelj & Zaversnik (2003) as in src/degeneracy.jl:38-96,
// with degree(g, v) = out + in degree for a digraph, whose in-neighbours are
// relaxed after the out-neighbours.  Returns -1 when a self-loop is present
// (the reference throws ArgumentError, :39).
int orc_core_number(int64_t n, const int64_t* rowptr, const int32_t* colidx,
                    const int64_t* in_rowptr, const int32_t* in_colidx, int directed,
                    int32_t* core) {
  if (directed && (!in_rowptr || !in_colidx)) return -1;
  for (int64_t v = 0; v < n; ++v)
    for (int64_t e = rowptr[v]; e < rowptr[v + 1]; ++e)
      if (colidx[e] == v) return -1;
  std::vector<int64_t> deg(n), pos(n), vert(n);
  int64_t maxdeg = 0;
  for (int64_t v = 0; v < n; ++v) {
    // degree(g, v): out + in for a digraph (src/core.jl:66)
    deg[v] = rowptr[v + 1] - rowptr[v] + (directed ? in_rowptr[v + 1] - in_rowptr[v] : 0);
    maxdeg = std::max(maxdeg, deg[v]);
  }
  std::vector<int64_t> bin(maxdeg + 1, 0);
  for (int64_t v = 0; v < n; ++v) bin[deg[v]]++;
  int64_t start = 0;
  for (int64_t d = 0; d <= maxdeg; ++d) {
    const int64_t num = bin[d];
    bin[d] = start;
    start += num;
  }
  for (int64_t v = 0; v < n; ++v) {
    pos[v] = bin[deg[v]];
    vert[pos[v]] = v;
    bin[deg[v]]++;
  }
  for (int64_t d = maxdeg; d >= 1; --d) bin[d] = bin[d - 1];
  if (maxdeg >= 0) bin[0] = 0;
  auto relax = [&](int64_t v, const int64_t* rp, const int32_t* ci) {
    for (int64_t e = rp[v]; e < rp[v + 1]; ++e) {
      const int64_t u = ci[e];
      if (deg[u] > deg[v]) {
        const int64_t du = deg[u], pu = pos[u], pw = bin[du], w = vert[pw];
        if (u != w) {
          pos[u] = pw;
          vert[pu] = w;
          pos[w] = pu;
          vert[pw] = u;
        }
        bin[du]++;
        deg[u]--;
      }
    }
  };
  for (int64_t i = 0; i < n; ++i) {
    const int64_t v = vert[i];
    relax(v, rowptr, colidx);                          // outneighbors, :63-79
    if (directed) relax(v, in_rowptr, in_colidx);      // inneighbors, :80-95
  }
  for (int64_t v = 0; v < n; ++v) core[v] = static_cast<int32_t>(deg[v]);
  return 0;
}

}  // extern "C"
