/* lgbc.h -- C ABI of the GB300-native betweenness-centrality / BFS library.
 *
 * This is the drop-in boundary for LightGraphs.jl's unit-weight betweenness
 * centrality and gdistances (LightGraphs v1.3.5; paths below are relative to
 * that project).  Host code (the Julia module in
 * lightgraphs.jl_gb300/julia/, or the Python mirror in
 * lightgraphs.jl_gb300/lgbc/) flattens SimpleGraph / SimpleDiGraph
 * `fadjlist` (and `badjlist`) to a 0-based CSR and calls these entry points;
 * every computation runs as hand-written sm_103a CUDA kernels.  There is no
 * CPU fallback: a missing or failing GPU is reported as an error.
 *
 * Conventions
 *  - Vertex ids are 0-based int32; rowptr is int64 (n+1 entries), colidx is
 *    int32 (nnz entries), each row sorted ascending without duplicates, as
 *    SimpleGraph's add_edge! keeps it (src/SimpleGraphs/simplegraph.jl:445-461,
 *    simpledigraph.jl:414-429).
 *  - The caller owns every host array.  The library copies what it needs to
 *    device memory before it returns and never keeps a host pointer.
 *  - Every entry point returns LGBC_OK (0) or a negative LGBC_E* code;
 *    lgbc_last_error() then returns a thread-local message.
 *  - A graph handle owns one CUDA stream.  Calls on one handle are serialised
 *    by a mutex; host-buffer calls are blocking (the stream is synchronised
 *    before they return).  "_dev" entry points are asynchronous on the
 *    handle's stream; lgbc_graph_sync() waits for them.
 */
#ifndef LGBC_H
#define LGBC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LGBC_OK 0
#define LGBC_EINVAL (-1)     /* bad vertex id, size or argument (ArgumentError/BoundsError) */
#define LGBC_ENOMEM (-2)     /* device or host allocation failed */
#define LGBC_ECUDA (-3)      /* a CUDA call failed (no GPU, launch failure, ...) */
#define LGBC_ETIMEOUT (-4)   /* a bounded device wait ran out; the context stays usable */

#define LGBC_UNREACHED INT32_MAX /* distance of a vertex no source reaches */

typedef struct lgbc_graph lgbc_graph; /* opaque; owns the device CSR */

/* Library version string, e.g. "lgbc 0.1.0 sm_103a". */
const char *lgbc_version(void);

/* Thread-local message describing the last error on this host thread. */
const char *lgbc_last_error(void);

/* Number of visible CUDA devices (0 if none); never fails. */
int lgbc_device_count(void);

/* Create a device-resident graph.
 * Replaces the per-call `g.fadjlist[u]` pointer chasing of
 * src/SimpleGraphs/SimpleGraphs.jl:78-79,93 (outneighbors) and
 * :85-86 (inneighbors) with one upload per graph.
 *   rowptr/colidx        out-CSR (fadjlist), nnz entries
 *   in_rowptr/in_colidx  in-CSR (badjlist) for directed graphs; NULL when
 *                        directed == 0 (an undirected graph is its own in-CSR)
 * A self-loop of an undirected graph is stored once, as add_edge! does
 * (src/SimpleGraphs/simplegraph.jl:455). */
int lgbc_graph_create(lgbc_graph **out, int64_t n, int64_t nnz,
                      const int64_t *rowptr, const int32_t *colidx,
                      const int64_t *in_rowptr, const int32_t *in_colidx,
                      int directed);

/* Free the handle and all its device memory. NULL is accepted. */
int lgbc_graph_destroy(lgbc_graph *g);

/* Number of vertices / stored CSR entries / directedness of a handle. */
int lgbc_graph_info(const lgbc_graph *g, int64_t *n, int64_t *nnz, int *directed);

/* gdistances!(g, sources, dists) -- src/traversals/bfs.jl:95-124,141 and the
 * Parallel variant src/Parallel/traversals/gdistances.jl:36-139.
 * Multi-source BFS: every source has distance 0, every other vertex the hop
 * count to the nearest source; LGBC_UNREACHED where no source reaches.
 * nsrc == 0 gives all LGBC_UNREACHED (test/traversals/bfs.jl:33). */
int lgbc_gdistances(lgbc_graph *g, const int32_t *src, int64_t nsrc,
                    int32_t *dist_out /* n */);

/* nsrc independent single-source gdistances, one per source, written as
 * dist_out[i * n + v] (row i = source i).  Runs sources as bit lanes of a
 * multi-source BFS that shares every edge read. */
int lgbc_gdistances_batch(lgbc_graph *g, const int32_t *src, int64_t nsrc,
                          int32_t *dist_out /* nsrc x n */);

/* Path counts and distances of dijkstra_shortest_paths(g, s) with unit
 * weights (src/shortestpaths/dijkstra.jl:59-141): DijkstraState.pathcounts
 * (:10, summed at :102,118, reset to 1 at the source at :135) and .dists,
 * for nsrc independent sources.  Row i (source src[i]) is
 *   sigma_out[i * n + v]  the number of shortest paths from src[i] to v as a
 *                         Float64: exact (the same bits as the reference's
 *                         sums) below 2^53, the exact count rounded to
 *                         nearest above; 1 at src[i]; 0 where src[i] does
 *                         not reach v
 *   dist_out[i * n + v]   hop distance, LGBC_UNREACHED where not reached
 *                         (dist_out may be NULL).
 * Counts are exact uint64 integers on the device; a batch whose counts could
 * pass 2^64 is recomputed with FP64 counts.  Sources run as bit lanes of the
 * multi-source BFS, 64 per batch. */
int lgbc_path_counts(lgbc_graph *g, const int32_t *src, int64_t nsrc, double *sigma_out,
                     int32_t *dist_out);

/* Unscaled Brandes betweenness over the given sources:
 * the source loop of src/centrality/betweenness.jl:46-68 (and of
 * Parallel.betweenness_centrality, src/Parallel/centrality/betweenness.jl:9-72)
 * with unit weights (DefaultDistance, src/distance.jl:8-21), i.e.
 * dijkstra_shortest_paths(allpaths=true) (src/shortestpaths/dijkstra.jl:59-141)
 * followed by _accumulate_basic! (:81-107) or, with endpoints != 0,
 * _accumulate_endpoints! (:109-134).  Sources with degree(g, s) == 0 are
 * skipped (:58; degree is in+out for digraphs, src/core.jl:66-67).
 * src == NULL means all vertices 0..n-1 (nsrc is then ignored).  Duplicate
 * sources are processed once per occurrence.  The caller applies _rescale!
 * (:136-160) with k = the number of sources passed (not the active count).
 * bc_raw_out: n doubles, overwritten. */
int lgbc_betweenness(lgbc_graph *g, const int32_t *src, int64_t nsrc,
                     int endpoints, double *bc_raw_out);

/* As lgbc_betweenness, but the result stays in device memory: bc_raw_dev is
 * a device pointer to n doubles (overwritten).  The source list is read from
 * host memory before the call returns; the computation is queued on the
 * handle's stream and may still run when the call returns. */
int lgbc_betweenness_dev(lgbc_graph *g, const int32_t *src, int64_t nsrc,
                         int endpoints, double *bc_raw_dev);

/* Exact betweenness (all sources) of many undirected graphs in one call:
 * betweenness_centrality(g) (src/centrality/betweenness.jl:46-75, before
 * _rescale!) for every graph g_i.  Graph i has n[i] vertices; its local
 * 0-based CSR is rowptr[rowptr_off[i] .. rowptr_off[i] + n[i]] (n[i] + 1
 * entries starting at 0) and colidx[col_off[i] ..] (local ids).  bc_raw_out
 * receives the graphs' raw vectors concatenated in input order (sum n[i]
 * doubles); the caller rescales each with _rescale!(bc_i, n[i], ...).
 * Graphs are grouped by size into disjoint unions; one 64-lane batch seeds
 * source index b*64 + l of every graph of a group in lane l, so each level
 * launch covers every graph of the group. */
int lgbc_betweenness_many(int64_t ngraphs, const int64_t *n, const int64_t *rowptr_off,
                          const int64_t *col_off, const int64_t *rowptr, const int32_t *colidx,
                          int endpoints, double *bc_raw_out);

/* Wait for all work queued on the handle's stream. */
int lgbc_graph_sync(lgbc_graph *g);

/* Device-side timing on the handle's stream: lgbc_timer_start records a CUDA
 * event, lgbc_timer_stop records a second one, synchronises, and returns the
 * elapsed milliseconds and the number of library kernels launched between
 * the two. */
int lgbc_timer_start(lgbc_graph *g);
int lgbc_timer_stop(lgbc_graph *g, double *elapsed_ms, int64_t *kernel_launches);

/* Statistics of the last betweenness / gdistances call on this handle. */
typedef struct lgbc_stats {
  int64_t kernel_launches;   /* kernels the call launched */
  int64_t batches;           /* source batches (<= 128 sources each) */
  int64_t levels;            /* BFS levels summed over batches */
  int64_t active_sources;    /* sources with degree > 0 */
  int64_t wide_batches;      /* batches replayed in FP64 because a path count exceeded 2^64 */
  int64_t topdown_levels;    /* levels expanded top-down */
  int64_t bottomup_levels;   /* levels expanded bottom-up */
} lgbc_stats;
int lgbc_graph_stats(const lgbc_graph *g, lgbc_stats *out);

/* Tunables (the autotuner writes these; defaults are used otherwise).
 *   alpha, beta   direction switch: go bottom-up when the frontier's edges
 *                 exceed (unvisited edges)/alpha; return top-down when the
 *                 frontier has fewer than n/beta vertices.
 *   hub_degree    vertices with more than this many neighbours ("hubs") are
 *                 cut into 256-edge work items spread over the whole GPU
 *                 instead of being expanded by one warp (default 256).
 *   lanes         sources per multi-source batch of the betweenness entry
 *                 points, stacked unions included (1..256, default 128; above
 *                 64 a batch keeps two 64-bit lane words per vertex, above 128
 *                 four); unions of many graphs use the default.  Stress and
 *                 distance batches use at most 64.
 *   dense_edges   a 32-edge chunk with more than this many edges that carry
 *                 lanes is gathered thread-per-lane (bit-transposed) instead
 *                 of edge by edge (32 = always edge by edge).
 *   segment_degree graphs whose mean degree (stored entries / n) is below
 *                 this run the low-degree kernels, in which a warp streams the
 *                 edges of 32 vertices at once (default 0 = never: on the
 *                 measured workloads the warp-per-vertex kernels were faster).
 *   source_order  1: before batching, sort the sources by their BFS distances
 *                 to the 16 highest-degree vertices (computed once per
 *                 graph), so that one batch holds sources with similar
 *                 distance profiles and reaches each vertex at fewer
 *                 distinct levels; 0: batch in the given order.  Results are
 *                 the same up to floating-point summation order.
 *   graph_loop    1: run each batch's level loops as CUDA graphs with
 *                 conditional nodes (the direction choice and the end of a
 *                 sweep are decided on the device; the host reads the control
 *                 block once per batch); 0: one host round trip per level.
 *   stack_vertices  small graphs run several source batches at once as a
 *                 disjoint union of R copies of the graph, each copy holding
 *                 its own batch of sources, with R * n <= stack_vertices
 *                 (used when R >= 4; 0 = never).  Default 2^21.
 *   hub_order     order of the hub work items: 0 hub by hub; 1 by the
 *                 neighbour id of each item's middle edge; 2 by the relative
 *                 position of each item in its hub's row (follows 1 on rows
 *                 sorted by neighbour id, without reading them on the host).
 *                 1 and 2 interleave the hubs so that the items in flight
 *                 gather rows of a limited range of vertices.  Default 2.
 *   dependency_df32  0: the dependency sums psi = (1 + delta) / sigma and
 *                 delta = sigma * sum(psi) are FP64, as the reference's
 *                 Float64 `coeff` and `delta` (src/centrality/betweenness.jl:
 *                 81-107) -- the default.  1: they are double-float (two
 *                 FP32 values, a 48-bit significand) -- faster on this GPU,
 *                 whose FP64 rate is a small fraction of its FP32 rate, and
 *                 still within 1e-9 of the FP64 result on the tested graphs,
 *                 but narrower than the reference's type.  Path counts are
 *                 exact uint64 integers either way (FP64 after an overflow).
 *                 Not changed by lgbc_tune. */
typedef struct lgbc_tuning {
  double alpha;
  double beta;
  int32_t hub_degree;
  int32_t lanes;
  int32_t dense_edges;
  int32_t segment_degree;
  int32_t source_order;
  int32_t graph_loop;
  int32_t stack_vertices;
  int32_t hub_order;
  int32_t dependency_df32;
} lgbc_tuning;
int lgbc_get_tuning(const lgbc_graph *g, lgbc_tuning *out);
int lgbc_set_tuning(lgbc_graph *g, const lgbc_tuning *t);

/* Autotuner (no counterpart in the reference).  Times Brandes passes over
 * 128 active sources spread over the vertex ids and picks, by coordinate
 * descent (two passes; a change must win by 2 %), the degree-bin cut
 * (hub_degree), the source-batch width (lanes), the direction-switch
 * thresholds (alpha, beta), the gather cuts (dense_edges, segment_degree) and
 * the hub item order (hub_order); the result stays set on the handle (read
 * it with lgbc_get_tuning).  Every setting gives the same results; only the
 * speed differs.  cache_path (may be NULL) is a text file of "signature alpha
 * beta hub_degree lanes dense_edges segment_degree source_order graph_loop
 * stack_vertices hub_order" lines, keyed by n, nnz, directedness and the device's SM
 * count: a matching line is applied without measuring, and a new result is
 * appended. */
int lgbc_tune(lgbc_graph *g, const char *cache_path);

/* gdistances for callers that cannot allocate device memory: no counterpart
 * in the reference.  The handle-based entry points copy the CSR to the device
 * and keep a BFS workspace, both from cudaMalloc.  Some callers cannot make
 * that call: a host whose device memory belongs to another allocator with a
 * fixed budget (a Julia CuArray pool, a serving process that reserves the
 * GPU's memory when it starts), where a cudaMalloc outside that allocator can
 * fail or take memory the budget counts on, and a loop that must not pay the
 * device-wide synchronisation cudaFree implies.  This entry point allocates
 * nothing.  Every input and output is a caller-owned DEVICE pointer: the CSR
 * (in_rowptr / in_colidx NULL for an undirected graph), the nsrc sources, and
 * dist (n int32, LGBC_UNREACHED where no source reaches).  Results equal
 * lgbc_gdistances'.  The BFS queue, frontier bitmaps and control block live in
 * one static device array of about 17 MB that every GPU which loads the
 * library holds until the process exits, so n is limited to
 * LGBC_NOALLOC_MAX_VERTICES (larger graphs get LGBC_EINVAL).  The CSR and the
 * sources are checked on the device before any kernel indexes with them
 * (rowptr running from 0 to nnz without decreasing, column ids and sources
 * in [0, n)); a bad input gets LGBC_EINVAL.  The first call on a device looks
 * up that array's address (cudaGetSymbolAddress) and the device's launch
 * shape; make that first call before any stream capture.  `stream` is a
 * cudaStream_t (NULL = default stream); the call synchronises that stream
 * after the check and after every BFS level, and returns when dist is
 * complete.  All calls share the one array, which keeps the last call's
 * contents (each call clears what must start at zero): calls that overlap on
 * the GPU (from several host threads or streams at once) race on it and must
 * not be issued. */
#define LGBC_NOALLOC_MAX_VERTICES (1 << 22)
int lgbc_gdistances_noalloc(int64_t n, int64_t nnz, const int64_t *rowptr,
                            const int32_t *colidx, const int64_t *in_rowptr,
                            const int32_t *in_colidx, const int32_t *src, int64_t nsrc,
                            int32_t *dist, void *stream);

/* ---- Learned source proposal (no counterpart in the reference) -----------
 *
 * Sampled betweenness with an importance-sampling proposal learned from
 * structure: raw(v) = sum_i w_i delta_{s_i}(v) with s_i drawn i.i.d. from p
 * and w_i = 1 / (k p_{s_i}), an unbiased estimate of the exact raw vector.
 * Passing it to _rescale!(raw, n, normalize, directed, n) gives the same
 * scale as betweenness_centrality(g) (uniform p = 1/n reproduces the n / k
 * factor of the k-sampled call).  p = (1 - eps) softmax(y) + eps / n, y the
 * output of a 4 -> 64 -> 64 -> 1 ReLU MLP over per-vertex features, trained
 * to predict log(1 + dependency mass).
 *
 * Undirected graphs only for the features and the proposal. */

/* Core numbers, as core_number(g) (src/degeneracy.jl:38-96; for a digraph
 * every arc counts at both ends, degree = out + in): LGBC_EINVAL for a graph
 * with a self-loop (the reference throws ArgumentError).  core_out: n int32. */
int lgbc_core_number(lgbc_graph *g, int32_t *core_out);

/* Per-vertex features, n x 4 float32 row-major: log(1 + degree),
 * log(1 + core number), mean of log(1 + degree) over the neighbours, and
 * log(1 + sum of the neighbours' degrees).  Degree = length(fadjlist[v]);
 * the core number is that of the graph without its self-loops. */
int lgbc_features(lgbc_graph *g, float *feat_out);

/* bfs_parents(g, s; dir) (src/traversals/bfs.jl:35-66): parents_out[v] is
 * the vertex from which the BFS from s first reaches v -- the smallest
 * neighbour one level closer, as the reference's sorted levels pick it --
 * parents_out[s] = s, and -1 where s does not reach (the reference's 0 in
 * 1-based ids).  dir 0 follows out-edges (:out), 1 in-edges (:in). */
int lgbc_bfs_parents(lgbc_graph *g, int32_t s, int dir, int32_t *parents_out);

/* has_path(g, u, v; exclude_vertices) (src/traversals/bfs.jl:150-172):
 * *result = 1 when v is reachable from u along out-edges without entering an
 * excluded vertex, or u == v; 0 when u or v is excluded or no path exists. */
int lgbc_has_path(lgbc_graph *g, int32_t u, int32_t v, const int32_t *exclude, int64_t nexclude,
                  int *result);

/* Stress centrality, unscaled, as stress_centrality(g, vs)
 * (src/centrality/stress.jl:33-77): for every source of degree > 0 the
 * reference's integer recursion over its shortest-path DAG, summed, in
 * wrapping Int64 arithmetic (bit-identical to Julia's, overflow included).
 * src NULL = every vertex; repeats count repeatedly.  stress_out: n int64. */
int lgbc_stress(lgbc_graph *g, const int32_t *src, int64_t nsrc, int64_t *stress_out);

/* Per-source BFS distance statistics (unit weights, along out-edges): for
 * source s_i, reached_out[i] = vertices reachable from s_i including itself,
 * dsum_out[i] = the sum of their distances, dmax_out[i] = the largest one
 * (any output may be NULL).  These are the reductions of the distance vector
 * of dijkstra_shortest_paths(g, s) (src/shortestpaths/dijkstra.jl:59-141)
 * that closeness_centrality (src/centrality/closeness.jl:33-55),
 * radiality_centrality (src/centrality/radiality.jl:36-49) and eccentricity
 * (src/distance.jl:73-79) take; the host finishes each metric from them.
 * Sources run as bit lanes of the multi-source BFS, 64 per batch. */
int lgbc_distance_stats(lgbc_graph *g, const int32_t *src, int64_t nsrc, int64_t *reached_out,
                        int64_t *dsum_out, int32_t *dmax_out);

/* Dependency mass of each source, mass_out[i] = sum_{v != s_i} delta_{s_i}(v):
 * the total that _accumulate_basic! (src/centrality/betweenness.jl:81-107)
 * adds to the betweenness vector for source s_i.  Computed exactly as
 * sum over reached t != s of (d(s, t) - 1), from the multi-source BFS. */
int lgbc_dependency_mass(lgbc_graph *g, const int32_t *src, int64_t nsrc, double *mass_out);

/* Weighted raw betweenness: bc_raw_out[v] = sum_i w[i] delta_{src[i]}(v)
 * (repeats allowed and merged into one traversal with the summed weight;
 * degree-0 sources contribute nothing).  endpoints=false accumulation only. */
int lgbc_betweenness_weighted(lgbc_graph *g, const int32_t *src, const double *w, int64_t nsrc,
                              double *bc_raw_out);

/* The MLP.  Parameters, in order: W1[64][4], b1[64], W2[64][64] (row = output
 * unit), b2[64], W3[64], b3 -- LGBC_MLP_PARAMS floats.  The network computes
 * with BF16 copies of FP32 master parameters and accumulates in FP32; inputs
 * are standardised as (x - mean) / stdev first. */
#define LGBC_MLP_FEATURES 4
#define LGBC_MLP_HIDDEN 64
#define LGBC_MLP_PARAMS 4545
typedef struct lgbc_mlp lgbc_mlp;
/* PyTorch-style uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) initialisation from
 * a seed; mean 0 / stdev 1 standardisation; fresh Adam state. */
int lgbc_mlp_create(lgbc_mlp **out, uint64_t seed);
int lgbc_mlp_destroy(lgbc_mlp *m);
/* master (LGBC_MLP_PARAMS float32) and / or bf16 (LGBC_MLP_PARAMS uint16 bit
 * patterns); either may be NULL. */
int lgbc_mlp_get_params(const lgbc_mlp *m, float *master, uint16_t *bf16);
/* Sets the master parameters (and their BF16 copies); resets Adam state. */
int lgbc_mlp_set_params(lgbc_mlp *m, const float *master);
int lgbc_mlp_set_norm(lgbc_mlp *m, const float *mean, const float *stdev);
int lgbc_mlp_get_norm(const lgbc_mlp *m, float *mean, float *stdev);
/* y[r] = MLP(x[r]) for rows x rows of 4 floats (host buffers). */
int lgbc_mlp_forward(lgbc_mlp *m, const float *x, int64_t rows, float *y);
/* Gradient (LGBC_MLP_PARAMS floats) and value of the centred squared error
 * (1/B) sum_r (e_r - mean e)^2, e_r = MLP(x_r) - target_r, over B = rows. */
int lgbc_mlp_grad(lgbc_mlp *m, const float *x, const float *target, int64_t rows, float *grad,
                  float *loss);
/* Adam training on the GPU.  Rows are grouped (group g = rows
 * [group_off[g], group_off[g + 1]), one graph each); every step takes one
 * group, chosen at random, and a random window of at most `batch` of its rows.
 * The learning rate warms up linearly over `warmup` steps, then decays by a
 * cosine to lr_final.  loss_out (steps floats, may be NULL) gets each step's
 * loss. */
typedef struct lgbc_train_cfg {
  int32_t steps;
  int32_t batch;
  int32_t warmup;
  float lr;
  float lr_final;
  float beta1;
  float beta2;
  float eps;
  uint64_t seed;
} lgbc_train_cfg;
int lgbc_mlp_train(lgbc_mlp *m, const float *x, const float *target, int64_t rows,
                   const int64_t *group_off, int64_t ngroups, const lgbc_train_cfg *cfg,
                   float *loss_out);

/* Build the proposal of graph g on the device: features, MLP scores, p and its
 * CDF (kept in the handle until the next build).  p_out (n doubles, may be
 * NULL) receives p. */
int lgbc_proposal_build(lgbc_graph *g, lgbc_mlp *m, double eps, double *p_out);
/* Draw k sources from the built proposal with weights 1 / (k p), seeded by
 * `seed` (SplitMix64).  LGBC_SAMPLE_IID: k independent draws.
 * LGBC_SAMPLE_SYSTEMATIC: systematic sampling on the CDF (draw i at
 * (i + U) / k, one uniform U), which draws source s floor or ceil of k p_s
 * times -- k p_s on average, so the weighted estimate stays unbiased -- with
 * lower variance.  Results come back in draw order (systematic draws in
 * vertex order). */
#define LGBC_SAMPLE_IID 0
#define LGBC_SAMPLE_SYSTEMATIC 1
int lgbc_proposal_sample(lgbc_graph *g, int64_t k, uint64_t seed, int scheme, int32_t *src_out,
                         double *w_out);

/* Graph ingest on the device: a handle built from a 0-based edge list
 * (src[i], dst[i]), i < m, with the storage semantics of add_edge! on
 * SimpleGraph / SimpleDiGraph (src/SimpleGraphs/simplegraph.jl:445-461,
 * simpledigraph.jl:414-429): neighbour lists sorted, duplicates dropped, an
 * undirected edge stored in both lists and an undirected self-loop once.  The
 * arcs are radix-sorted on the GPU; only the edge list crosses to the device.
 * LGBC_EINVAL for an endpoint outside [0, n). */
int lgbc_graph_create_from_edges(lgbc_graph **out, int64_t n, int64_t m, const int32_t *src,
                                 const int32_t *dst, int directed);
/* Copy a handle's CSR to the host: rowptr (n + 1 int64), colidx (nnz int32)
 * and, for a digraph, the in-CSR; any pointer may be NULL (nnz from
 * lgbc_graph_info). */
int lgbc_graph_csr(const lgbc_graph *g, int64_t *rowptr, int32_t *colidx, int64_t *in_rowptr,
                   int32_t *in_colidx);

/* Device / pinned-host memory helpers for callers without their own CUDA
 * allocator (bench and test harnesses).  lgbc_memcpy kinds: 1 = host to
 * device, 2 = device to host, 3 = device to device. */
int lgbc_device_alloc(void **ptr, int64_t bytes);
int lgbc_device_free(void *ptr);
int lgbc_host_alloc(void **ptr, int64_t bytes);
int lgbc_host_free(void *ptr);
int lgbc_memcpy(void *dst, const void *src, int64_t bytes, int kind);

#ifdef __cplusplus
}
#endif

#endif /* LGBC_H */
