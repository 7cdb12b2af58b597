// generators.cpp -- seeded host-side generators of the benchmark / test graphs
// (declared in include/lgbc_gen.h).  Not on the GPU path.
#include "lgbc_gen.h"

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <unordered_set>
#include <vector>

namespace {

// SplitMix64 (Steele, Lea & Flood 2014): a 64-bit counter passed through a
// bijective mixing function.
inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct SplitMix {
  uint64_t state;
  explicit SplitMix(uint64_t seed) : state(seed) {}
  uint64_t next() {
    state += 0x9E3779B97F4A7C15ull;
    return mix64(state);
  }
  double uniform() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }
  uint64_t below(uint64_t m) {  // uniform in [0, m)
    return static_cast<uint64_t>((static_cast<unsigned __int128>(next()) * m) >> 64);
  }
};

// Independent stream per (seed, stream id).
inline SplitMix stream(uint64_t seed, uint64_t id) {
  return SplitMix(mix64(seed * 0x9E3779B97F4A7C15ull + mix64(id + 0x632BE59BD9B4E019ull)));
}

int hw_threads() {
  unsigned t = std::thread::hardware_concurrency();
  return static_cast<int>(std::max(1u, std::min(t, 64u)));
}

template <class Fn>
void parallel_for(int64_t count, Fn fn) {
  const int T = hw_threads();
  if (T <= 1 || count < 4096) {
    fn(0, count, 0);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < T; ++t) {
    const int64_t lo = count * t / T, hi = count * (t + 1) / T;
    th.emplace_back([=, &fn]() { fn(lo, hi, t); });
  }
  for (auto& x : th) x.join();
}

// Sort keys in [0, keyspace) with a parallel bucket pass + per-bucket sorts,
// then drop duplicates.
void sort_unique(std::vector<uint64_t>& keys, uint64_t keyspace) {
  const int64_t N = static_cast<int64_t>(keys.size());
  const int T = hw_threads();
  if (N < (1 << 16) || T <= 1) {
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    return;
  }
  const uint64_t nb = static_cast<uint64_t>(T) * 64;
  auto bucket = [&](uint64_t k) {
    return static_cast<uint64_t>((static_cast<unsigned __int128>(k) * nb) / keyspace);
  };
  std::vector<std::vector<int64_t>> cnt(T, std::vector<int64_t>(nb + 1, 0));
  parallel_for(N, [&](int64_t lo, int64_t hi, int t) {
    for (int64_t i = lo; i < hi; ++i) cnt[t][bucket(keys[i])]++;
  });
  // exclusive offsets: bucket-major, thread-minor
  std::vector<std::vector<int64_t>> off(T, std::vector<int64_t>(nb, 0));
  std::vector<int64_t> bstart(nb + 1, 0);
  int64_t acc = 0;
  for (uint64_t b = 0; b < nb; ++b) {
    bstart[b] = acc;
    for (int t = 0; t < T; ++t) {
      off[t][b] = acc;
      acc += cnt[t][b];
    }
  }
  bstart[nb] = acc;
  std::vector<uint64_t> out(keys.size());
  parallel_for(N, [&](int64_t lo, int64_t hi, int t) {
    for (int64_t i = lo; i < hi; ++i) out[off[t][bucket(keys[i])]++] = keys[i];
  });
  std::atomic<uint64_t> nextb(0);
  std::vector<std::thread> th;
  for (int t = 0; t < T; ++t)
    th.emplace_back([&]() {
      for (;;) {
        uint64_t b = nextb.fetch_add(1);
        if (b >= nb) break;
        std::sort(out.begin() + bstart[b], out.begin() + bstart[b + 1]);
      }
    });
  for (auto& x : th) x.join();
  out.erase(std::unique(out.begin(), out.end()), out.end());
  keys.swap(out);
}

// CSR from sorted unique keys u * n + v.
void csr_from_keys(const std::vector<uint64_t>& keys, int64_t n, int64_t** rowptr, int32_t** colidx) {
  const int64_t nnz = static_cast<int64_t>(keys.size());
  int64_t* rp = static_cast<int64_t*>(std::malloc(sizeof(int64_t) * (n + 1)));
  int32_t* ci = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * std::max<int64_t>(nnz, 1)));
  std::fill(rp, rp + n + 1, 0);
  for (int64_t i = 0; i < nnz; ++i) rp[keys[i] / n + 1]++;
  for (int64_t v = 0; v < n; ++v) rp[v + 1] += rp[v];
  parallel_for(nnz, [&](int64_t lo, int64_t hi, int) {
    for (int64_t i = lo; i < hi; ++i) ci[i] = static_cast<int32_t>(keys[i] % n);
  });
  *rowptr = rp;
  *colidx = ci;
}

// Fill `out` from a list of edges given as keys (undirected: lo * n + hi,
// lo < hi; directed: u * n + v), sorted and unique.
int finish(std::vector<uint64_t>& edges, int64_t n, int directed, lgbc_csr* out) {
  std::memset(out, 0, sizeof(*out));
  out->n = n;
  out->m = static_cast<int64_t>(edges.size());
  out->directed = directed ? 1 : 0;
  const uint64_t space = static_cast<uint64_t>(n) * static_cast<uint64_t>(n);
  if (!directed) {
    std::vector<uint64_t> both(edges.size() * 2);
    parallel_for(static_cast<int64_t>(edges.size()), [&](int64_t lo, int64_t hi, int) {
      for (int64_t i = lo; i < hi; ++i) {
        const uint64_t a = edges[i] / n, b = edges[i] % n;
        both[2 * i] = a * n + b;
        both[2 * i + 1] = b * n + a;
      }
    });
    std::vector<uint64_t>().swap(edges);
    sort_unique(both, space);
    out->nnz = static_cast<int64_t>(both.size());
    csr_from_keys(both, n, &out->rowptr, &out->colidx);
  } else {
    out->nnz = static_cast<int64_t>(edges.size());
    csr_from_keys(edges, n, &out->rowptr, &out->colidx);
    std::vector<uint64_t> rev(edges.size());
    parallel_for(static_cast<int64_t>(edges.size()), [&](int64_t lo, int64_t hi, int) {
      for (int64_t i = lo; i < hi; ++i) rev[i] = (edges[i] % n) * n + edges[i] / n;
    });
    sort_unique(rev, space);
    csr_from_keys(rev, n, &out->in_rowptr, &out->in_colidx);
  }
  return 0;
}

}  // namespace

extern "C" {

int lgbc_gen_rmat(int scale, int edgefactor, double a, double b, double c, uint64_t seed,
                  int directed, lgbc_csr* out) {
  if (!out || scale < 1 || scale > 30 || edgefactor < 1 || a <= 0 || b < 0 || c < 0 ||
      a + b + c >= 1.0)
    return -1;
  const int64_t N = int64_t(1) << scale;
  const int64_t M = static_cast<int64_t>(edgefactor) * N;
  const double ab = a + b;
  const double c_norm = c / (1.0 - ab);
  const double a_norm = a / ab;
  // random permutation of the vertex ids (Fisher-Yates)
  std::vector<int64_t> perm(N);
  for (int64_t i = 0; i < N; ++i) perm[i] = i;
  {
    SplitMix r = stream(seed, ~0ull);
    for (int64_t i = N - 1; i > 0; --i) std::swap(perm[i], perm[r.below(i + 1)]);
  }
  std::vector<uint64_t> keys(M);
  std::vector<char> keep(M);
  parallel_for(M, [&](int64_t lo, int64_t hi, int) {
    for (int64_t e = lo; e < hi; ++e) {
      SplitMix r = stream(seed, static_cast<uint64_t>(e));
      int64_t i = 0, j = 0;
      for (int ib = 0; ib < scale; ++ib) {
        const bool ii = r.uniform() > ab;
        const bool jj = r.uniform() > (ii ? c_norm : a_norm);
        i |= static_cast<int64_t>(ii) << ib;
        j |= static_cast<int64_t>(jj) << ib;
      }
      const int64_t u = perm[i], v = perm[j];
      keep[e] = u != v;
      if (directed) {
        keys[e] = static_cast<uint64_t>(u) * N + v;
      } else {
        const int64_t lo_ = std::min(u, v), hi_ = std::max(u, v);
        keys[e] = static_cast<uint64_t>(lo_) * N + hi_;
      }
    }
  });
  int64_t w = 0;
  for (int64_t e = 0; e < M; ++e)
    if (keep[e]) keys[w++] = keys[e];
  keys.resize(w);
  std::vector<char>().swap(keep);
  sort_unique(keys, static_cast<uint64_t>(N) * N);
  return finish(keys, N, directed, out);
}

int lgbc_gen_erdos_renyi(int64_t n, int64_t m, uint64_t seed, int directed, lgbc_csr* out) {
  if (!out || n < 1 || m < 0) return -1;
  const long double maxe = directed ? static_cast<long double>(n) * (n - 1)
                                    : static_cast<long double>(n) * (n - 1) / 2;
  if (m > maxe * 2 / 3) return -1;
  SplitMix r = stream(seed, 0);
  std::unordered_set<uint64_t> seen;
  seen.reserve(static_cast<size_t>(m) * 2);
  std::vector<uint64_t> keys;
  keys.reserve(static_cast<size_t>(m));
  while (static_cast<int64_t>(keys.size()) < m) {
    const int64_t u = static_cast<int64_t>(r.below(n));
    const int64_t v = static_cast<int64_t>(r.below(n));
    if (u == v) continue;
    uint64_t key;
    if (directed) key = static_cast<uint64_t>(u) * n + v;
    else key = static_cast<uint64_t>(std::min(u, v)) * n + std::max(u, v);
    if (seen.insert(key).second) keys.push_back(key);
  }
  std::sort(keys.begin(), keys.end());
  return finish(keys, n, directed, out);
}

int lgbc_gen_barabasi_albert(int64_t n, int k, uint64_t seed, lgbc_csr* out) {
  if (!out || k < 1 || n < k) return -1;
  SplitMix r = stream(seed, 0);
  int64_t n0 = k;
  std::vector<uint64_t> keys;
  keys.reserve(static_cast<size_t>((n - n0) * k));
  std::vector<int64_t> weighted;
  weighted.reserve(static_cast<size_t>(2 * (n - n0) * k + 2 * k));
  if (n0 < n) {
    // the graph has no edges: vertex n0 joins all k seed vertices
    // (sample!(rng, 1:n0, k) draws all of them when n0 == k)
    for (int64_t t = 0; t < n0; ++t) {
      keys.push_back(static_cast<uint64_t>(t) * n + n0);
      weighted.push_back(t);
      weighted.push_back(n0);
    }
    n0 += 1;
  }
  std::vector<char> picked(static_cast<size_t>(n), 0);
  std::vector<int64_t> targets(static_cast<size_t>(k));
  for (int64_t source = n0; source < n; ++source) {
    int i = 0;
    while (i < k) {
      const int64_t t = weighted[r.below(weighted.size())];
      if (!picked[t]) {
        targets[i++] = t;
        picked[t] = 1;
      }
    }
    for (int j = 0; j < k; ++j) {
      const int64_t t = targets[j];
      keys.push_back(static_cast<uint64_t>(std::min(t, source)) * n + std::max(t, source));
      weighted.push_back(source);
      weighted.push_back(t);
      picked[t] = 0;
    }
  }
  std::sort(keys.begin(), keys.end());
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  return finish(keys, n, 0, out);
}

void lgbc_csr_free(lgbc_csr* g) {
  if (!g) return;
  std::free(g->rowptr);
  std::free(g->colidx);
  std::free(g->in_rowptr);
  std::free(g->in_colidx);
  std::memset(g, 0, sizeof(*g));
}

}  // extern "C"
