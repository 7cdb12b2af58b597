// lgbc_kernels.h -- host-side launch wrappers shared by the CUDA translation
// units of the lgbc library.  Every wrapper returns the number of kernels it
// queued, which the API layer counts for lgbc_stats / lgbc_timer_stop.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "lgbc_internal.cuh"

struct lgbc_mlp;

namespace lgbc {

// Path-count representation of a multi-source batch.
enum SigmaKind : int {
  kSigmaNone = 0,    // distances only (gdistances_batch)
  kSigmaU64 = 1,     // exact uint64 path counts, double-float (df32) dependency sums (opt-in)
  kSigmaF64 = 2,     // FP64 path counts and dependencies (replay after overflow)
  kSigmaU64F64 = 3,  // exact uint64 path counts, FP64 dependencies (the default)
};
// The forward sweep only sees the path counts: both uint64 kinds run the same
// forward kernels.
constexpr int fwd_kind(int sk) { return sk == kSigmaU64F64 ? kSigmaU64 : sk; }
// Path counts kept as exact uint64 (an overflow replays the batch in FP64).
constexpr bool u64_counts(int sk) { return sk == kSigmaU64 || sk == kSigmaU64F64; }

// Landmark vertices (highest degree) whose BFS distances order the sources.
constexpr int kLandmarks = 16;

struct LaunchCfg {
  int grid;     // blocks for grid-stride kernels
  int block;    // threads per block
  int sms;      // streaming multiprocessors on the device
};

// ---- multi-source (bit-lane) BFS and Brandes sweeps: msbfs.cu ----------
// Per-batch device buffers.  A batch has 64 * words lanes (words = 1 or 2);
// every lane set is `words` consecutive uint64 (lane l in word l / 64, bit
// l % 64), so the mask of vertex v is at [v * words], and lane l of v's
// path-count / psi row lives at [v * 64 * words + l].  The buffers are sized
// for two words; a one-word batch uses their first half.
struct MsBuffers {
  uint64_t* visit;     // n lane sets: lanes that have reached v
  uint64_t* mb[2];     // n lane sets each: dense level masks, F_L lives in mb[L & 1]
  void* sigma;         // n rows: uint64 or double path counts
  void* psi;           // n rows: df32 or double, (1 + delta) / sigma
  int32_t* qv;         // cap: concatenated level lists (vertex)
  uint64_t* qm;        // cap lane sets: lanes of that vertex at that level
  unsigned long long* lvl_off;  // n + 3: start of each level's list
  BatchCtl* ctl;       // control block
  const int32_t* lane_src;      // sources of the batch (device)
  unsigned long long cap;       // entries in qv / qm
  const double* lane_w;         // 64 * words lane weights (weighted accumulation) or nullptr
  int64_t lane_w_n;             // > 0: a union of copies of an n-vertex graph, one row of 64
                                // weights per copy (vertex v uses row v / lane_w_n; one word)
  unsigned* claim;              // n, two-word batches: top-down first-discovery flags, kept zero
  int words;                    // 64-bit lane words per vertex: 1 or 2
  int lane_filter;              // 1: bottom-up levels skip lanes absent from the frontier
};

// The active lanes of a batch (word 1 unused in a one-word batch).
struct LaneSet {
  uint64_t w[kMaxWords];
};
// Lanes [0, nl) of a batch with `words` words.
inline LaneSet lane_set(int nl, int words) {
  LaneSet a{};
  for (int j = 0; j < words; ++j) {
    const int k = nl - 64 * j;
    a.w[j] = k >= 64 ? ~0ull : (k <= 0 ? 0ull : ((1ull << k) - 1ull));
  }
  return a;
}

// Vertices with more than hub_degree neighbours ("hubs") are not expanded by
// one warp: their edge lists are cut into kHubChunk-edge work items spread over
// the whole grid, whose partial results are combined with atomics; the last
// item of a hub to finish (a completion counter, no waiting) finalises it.
constexpr int kHubChunk = 256;
struct HubItem {
  int64_t lo, hi;      // edge range [lo, hi) in the CSR the item list belongs to
  int32_t v;           // the hub vertex
  int32_t slot;        // its accumulator slot
  int32_t nitems;      // items of this hub in this list
  int32_t pad;
};
struct HubData {
  const HubItem* out_items;      // items over out-edges (top-down discovery, dependencies)
  long long n_out;
  const HubItem* in_items;       // items over in-edges (path-count pulls, bottom-up)
  long long n_in;
  unsigned long long* acc;       // slots x 64 * words partial sums (uint64 or FP64 bits), kept zero
  unsigned long long* mask;      // slots x words: OR of discovering lanes, kept zero
  unsigned int* cnt;             // slots: finished items, kept zero
  int hub_degree;                // degree above which a vertex is a hub (INT32_MAX: none)
  int dense_edges;               // chunks with more contributing edges use the transposed gather
  int segmented;                 // 1: low-degree kernels (a warp streams 32 vertices' edges)
};

// sigma_limit: (2^64 - 1) / (max in-degree + 1), the largest path count a
// level may hold without the next level risking 64-bit overflow.
int ms_init(cudaStream_t s, const DevGraph& g, const MsBuffers& b, int nlanes, int sigma_kind,
            unsigned long long sigma_limit, int32_t* dist, int64_t dist_ld);
// Level 0 from explicit (vertex, lane set) seeds (distinct vertices; b.words
// mask words per seed); for disjoint unions of graphs, where one lane holds a
// source in every component.  Distances (dist) only with one word.
int ms_init_seeds(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const MsBuffers& b,
                  const int32_t* seed_v, const uint64_t* seed_mask, int64_t nseeds, int sigma_kind,
                  unsigned long long sigma_limit, int32_t* dist, int64_t dist_ld);
// visit[v] = seg_mark[k] (b.words words) for every vertex of segment k
// (vertices [seg_off[k], seg_off[k+1])): the lanes with no source in that
// component.
int ms_premark(const LaunchCfg& c, cudaStream_t s, const MsBuffers& b, const int64_t* seg_off,
               const uint64_t* seg_mark, int64_t nseg);
// Top-down / bottom-up level.  Distances (dist) only with one word.
int ms_topdown(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const MsBuffers& b,
               const HubData& hd, const LaneSet& act, int sigma_kind, int32_t* dist,
               int64_t dist_ld);
int ms_bottomup(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const MsBuffers& b,
                const HubData& hd, const LaneSet& act, int sigma_kind, int32_t* dist,
                int64_t dist_ld);
int ms_advance(cudaStream_t s, const DevGraph& g, const MsBuffers& b);
// Set ctl->level = maxlevel for the backward sweep (on the device).
int ms_begin_backward(cudaStream_t s, const MsBuffers& b);
// Backward (dependency) step for the level in ctl->level, then level--.
int ms_backward_level(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const MsBuffers& b,
                      const HubData& hd, int sigma_kind, double* bc);
// The same without the final level decrement (the body of a device-driven loop).
int ms_backward_body(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const MsBuffers& b,
                     const HubData& hd, int sigma_kind, double* bc);

// Device-driven level loops: the control kernels of a CUDA graph whose
// conditional nodes run the forward levels (WHILE `loop` { SWITCH `dir` })
// and the backward levels (WHILE `loop`).
struct LoopParams {
  cudaGraphConditionalHandle loop;  // 1: run another iteration
  cudaGraphConditionalHandle dir;   // forward: 0 top-down, 1 bottom-up, 2 none
  long long n;
  long long nnz;
  double alpha;                     // direction-switch thresholds
  double beta;
  int sigma_kind;
  long long max_levels;             // runaway cap (n + 1)
};
int loop_arm(cudaStream_t s, const MsBuffers& b, const LoopParams& lp);
int loop_advance(cudaStream_t s, const MsBuffers& b, const LoopParams& lp);
int loop_back_arm(cudaStream_t s, const MsBuffers& b, const LoopParams& lp);
int loop_back_advance(cudaStream_t s, const MsBuffers& b, const LoopParams& lp);
// Stress step for the level in ctl->level after a distance-only forward
// sweep (E = 1 + D per (vertex, lane) in the path-count rows), adding the
// stress of level + 1 into `stress` (wrapping uint64); then level--.
int st_backward_level(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const MsBuffers& b,
                      const HubData& hd, unsigned long long* stress);
// After the backward sweep: clear the masks of levels 0 and 1.
int ms_cleanup(const LaunchCfg& c, cudaStream_t s, const MsBuffers& b);
// Per-lane distance statistics of a batch (64 entries each, accumulated):
// vertices reached at levels >= 1, the sum of their levels, the deepest level.
struct LevelStats {
  unsigned long long* cnt;
  unsigned long long* dsum;
  int* dmax;
};
// After a distance-only forward sweep (before ms_cleanup_all).
int ms_level_stats(const LaunchCfg& c, cudaStream_t s, const MsBuffers& b, const LevelStats& st);
// After a distance-only batch: clear visit / masks of every listed vertex.
int ms_cleanup_all(const LaunchCfg& c, cudaStream_t s, const MsBuffers& b);
// After the forward sweep of a one-word batch with path counts (uint64 or
// FP64 kind): sigma_out[l * ld + v] = path count of lane l at v as binary64,
// dist_out[l * ld + v] = its level (dist_out may be null), for every listed
// (vertex, lane); unlisted entries are left as they are.
int ms_export(const LaunchCfg& c, cudaStream_t s, const MsBuffers& b, int sigma_kind,
              double* sigma_out, int32_t* dist_out, int64_t ld);
// Zero visit and both mask buffers outright (after an aborted batch).
int ms_reset_all(cudaStream_t s, const DevGraph& g, const MsBuffers& b);

// ---- single multi-source BFS (gdistances): bfs.cu ------------------------
struct BfsBuffers {
  int32_t* queue;               // n: every level, concatenated
  uint32_t* bm[2];              // (n + 31) / 32 words each: frontier bitmaps
  BatchCtl* ctl;
  int32_t* large = nullptr;     // n or null: frontier vertices with more than kBfsLarge
                                // out-edges, expanded by the whole grid (null: by one warp)
};
constexpr int kBfsLarge = 1024;
int bfs_init(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const BfsBuffers& b,
             const int32_t* src, int64_t nsrc, int32_t* dist);
int bfs_topdown(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const BfsBuffers& b,
                int32_t* dist);
int bfs_bottomup(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const BfsBuffers& b,
                 int32_t* dist, int stage_smem);
int bfs_advance(cudaStream_t s, const BfsBuffers& b);
// parents[v] = smallest in-neighbour of v at distance dist[v] - 1 (the
// source: itself; unreached: -1).
int bfs_parents(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const int32_t* dist,
                int32_t* parents);
// p[idx[i]] = value for i < count.
int scatter_i32(const LaunchCfg& c, cudaStream_t s, int32_t* p, const int32_t* idx, int64_t count,
                int32_t value);
// Largest dynamic shared memory the bottom-up kernel may stage (bytes).
int bfs_configure(size_t max_dyn_smem);

// Set the thread-local message returned by lgbc_last_error() (api.cu).
void set_last_error(const char* msg);

// ---- small utilities: util.cu ----------------------------------------------
// ORs into *bad: 1 = rowptr decreases somewhere, 2 = a column index is not in
// [0, n), 4 = rowptr[0] != 0 or rowptr[n] != nnz.
int validate_csr(const LaunchCfg& c, cudaStream_t s, const int64_t* rowptr, const int32_t* colidx,
                 int64_t n, int64_t nnz, int* bad);
int fill_i32(const LaunchCfg& c, cudaStream_t s, int32_t* p, int64_t count, int32_t value);
// The CSR of a disjoint union of `copies` copies of an n-vertex graph (copy
// r = vertices [r n, (r + 1) n)): rp1[copies n + 1], c1[copies nnz]; n > 0.
int replicate_csr(const LaunchCfg& c, cudaStream_t s, const int64_t* rp0, const int32_t* c0,
                  int64_t n, int64_t nnz, int64_t copies, int64_t* rp1, int32_t* c1);
// out[v] = sum over r < copies of stacked[r * n + v] (a fixed order).
int sum_copies(const LaunchCfg& c, cudaStream_t s, const double* stacked, int64_t n, int64_t copies,
               double* out);
// out[r * nl + j] = dist[j * ld + src[r]] for r < k, j < nl.
int gather_cols(const LaunchCfg& c, cudaStream_t s, const int32_t* dist, int64_t ld, int nl,
                const int32_t* src, int64_t k, int32_t* out);
int fill_f64(const LaunchCfg& c, cudaStream_t s, double* p, int64_t count, double value);
// bc[v] += k_act for every v, then bc[s] += n - 2 for each active source s:
// the endpoint terms of _accumulate_endpoints! summed over the sources.
int add_endpoints(const LaunchCfg& c, cudaStream_t s, double* bc, int64_t n,
                  const int32_t* active_src, int64_t k_act);
// The same for a disjoint union of graphs: segment i = vertices [seg_off[i],
// seg_off[i+1]) gets seg_add[i] (its active-source count) everywhere, and each
// active source src[j] gets src_add[j] (its graph's n - 2) more.
int add_endpoints_many(const LaunchCfg& c, cudaStream_t s, double* bc, const int64_t* seg_off,
                       const double* seg_add, int64_t nseg, const int32_t* src,
                       const double* src_add, int64_t nsrc);

// ---- learned source proposal: learned.cu ----------------------------------
// deg[v] = neighbours other than v; *loops |= 1 if v has a self-loop.
int core_degree(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, int32_t* deg, int* loops);
// One h-index pass over list[0, nlist) (all vertices when list is null):
// lowered vertices are logged (vertex, old value) -- those with more than 256
// neighbour entries ("hubs", deferred to `large` and searched by a block each)
// in the hub log -- and then their neighbours whose count can have changed
// are flagged.  Every array holds n entries.
struct CorePassBuffers {
  unsigned long long* changed;       // lowered non-hub vertices this pass
  unsigned long long* changed_hubs;  // lowered hubs this pass
  unsigned long long* nlarge;        // hubs deferred this pass
  int32_t* log_v;
  int32_t* log_old;
  int32_t* hub_v;
  int32_t* hub_old;
  int32_t* large;
};
int core_pass(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const int32_t* list,
              int64_t nlist, int32_t* core, uint8_t* flag, const CorePassBuffers& b);
// list <- flagged vertices (flags cleared), *count += their number.
int core_compact(const LaunchCfg& c, cudaStream_t s, int64_t n, uint8_t* flag, int32_t* list,
                 unsigned long long* count);
int features(const LaunchCfg& c, cudaStream_t s, const DevGraph& g, const int32_t* core,
             float4* feat);

// MLP parameter layout (floats): W1[64][4], b1[64], W2[64][64], b2[64], W3[64], b3.
constexpr int kMlpHidden = 64;
constexpr int kMlpW1 = 0;
constexpr int kMlpB1 = kMlpW1 + kMlpHidden * 4;
constexpr int kMlpW2 = kMlpB1 + kMlpHidden;
constexpr int kMlpB2 = kMlpW2 + kMlpHidden * kMlpHidden;
constexpr int kMlpW3 = kMlpB2 + kMlpHidden;
constexpr int kMlpB3 = kMlpW3 + kMlpHidden;
constexpr int kMlpParams = kMlpB3 + 1;                  // 4545
constexpr int kMlpParamsPadded = (kMlpParams + 3) & ~3;
constexpr int kGradRows = kMlpHidden;                   // rows per gradient block
constexpr int kGradThreads = 2 * kMlpHidden;            // two threads per row
static_assert(kMlpParams == 4545, "parameter count");

struct MlpNorm {
  float mu[4];
  float isd[4];   // 1 / stdev
};
struct AdamStep {
  float lr, beta1, beta2, eps;
  float bc1, bc2;  // bias corrections 1 - beta^t
};
int mlp_forward(const LaunchCfg& c, cudaStream_t s, const float4* x, int64_t rows,
                const __nv_bfloat16* P, const MlpNorm& nm, float* y);
// Opt the gradient kernel into its dynamic shared memory (once per device).
int mlp_configure();
// One step on rows [r0, r0 + B): residuals e, their mean (center, one
// float), block partials part, the loss, the reduced gradient (grad may be
// null) and, when master is not null, an Adam update of master / Pw / m1 / m2.
int mlp_train_step(cudaStream_t s, const float4* x, const float* target, int64_t r0, int B,
                   const __nv_bfloat16* P, const MlpNorm& nm, float* e, float* center,
                   float* part, float* loss, float* grad, float* master, __nv_bfloat16* Pw,
                   float* m1, float* m2, const AdamStep& st);
int mlp_to_bf16(cudaStream_t s, const float* master, __nv_bfloat16* P);
// Weights and standardisation of an MLP handle (mlp.cu), for graph calls.
struct MlpView {
  const __nv_bfloat16* P;
  MlpNorm norm;
  int device;
};
int mlp_view(const lgbc_mlp* m, MlpView* out);

// Proposal scratch: tiles of the scan; fscratch needs tiles + 1 floats, tsum
// tiles doubles, scal 1 double.
int64_t proposal_tiles(int64_t n);
int proposal_build(cudaStream_t s, const float* y, int64_t n, double eps, float* fscratch,
                   double* e, double* tsum, double* scal, double* p, double* cdf);
// systematic: draw i uses u_i = (i + U) / k with one uniform U, else k
// independent uniforms.
int proposal_sample(cudaStream_t s, const double* cdf, const double* p, int64_t n, int64_t k,
                    uint64_t seed, bool systematic, int32_t* src, double* w);

// ---- graph ingest on the device: ingest.cu -------------------------------------
// Bit width B of the vertex ids in the 64-bit arc keys (u << B) | v.
int ingest_bits(int64_t n);
// Scan tiles (int64 partial sums needed) for a scan of `count` items.
int64_t scan_tiles(int64_t count);
// Arc keys of an edge list (2 per edge for an undirected graph; a self-loop
// keeps one); *bad |= 1 for ids outside [0, n).
int ingest_make_keys(const LaunchCfg& c, cudaStream_t s, const int32_t* src, const int32_t* dst,
                     int64_t m, int64_t n, int B, int directed, unsigned long long* keys, int* bad);
int ingest_swap_keys(const LaunchCfg& c, cudaStream_t s, const unsigned long long* in, int64_t count,
                     int B, unsigned long long* out);
// Histogram cells of a radix sort of `count` keys (hist: uint32, off: int64 each).
int64_t radix_scratch_words(int64_t count);
// LSD radix sort of the low `bits` bits; keys / alt are swapped as passes run
// (on return `keys` holds the sorted keys).
int radix_sort(cudaStream_t s, unsigned long long*& keys, unsigned long long*& alt, int64_t count,
               int bits, uint32_t* hist, int64_t* off, int64_t* sums);
// keep[i] = first copy of key i (no sentinel); pos = exclusive scan; *nkept.
int ingest_unique(const LaunchCfg& c, cudaStream_t s, const unsigned long long* keys, int64_t count,
                  uint8_t* keep, int64_t* pos, int64_t* sums, int64_t* nkept);
int ingest_emit(const LaunchCfg& c, cudaStream_t s, const unsigned long long* keys, int64_t count,
                const uint8_t* keep, const int64_t* pos, int B, int32_t* colidx, unsigned int* deg);
int ingest_compact(const LaunchCfg& c, cudaStream_t s, const unsigned long long* keys, int64_t count,
                   const uint8_t* keep, const int64_t* pos, unsigned long long* out);
// rowptr[0..n] from the row lengths.
int ingest_rowptr(cudaStream_t s, const unsigned int* deg, int64_t n, int64_t* sums, int64_t* rowptr);

}  // namespace lgbc
