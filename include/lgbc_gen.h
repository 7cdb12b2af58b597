/* lgbc_gen.h -- seeded graph generators for the workloads of this library.
 *
 * Host-only helpers exported by liblgbc.so.  They are not on the GPU path and
 * have no counterpart in the C ABI a LightGraphs binding needs; they build
 * the benchmark and test inputs with the semantics of LightGraphs' own
 * generators (LightGraphs v1.3.5, src/SimpleGraphs/generators/randgraphs.jl).
 * Julia's MersenneTwister stream cannot be reproduced here, so the graphs are
 * distributionally -- not bit-for-bit -- those of the reference generators.
 * Randomness: SplitMix64 (Steele, Lea & Flood, OOPSLA 2014) keyed by
 * (seed, draw index), so results do not depend on the thread count.
 */
#ifndef LGBC_GEN_H
#define LGBC_GEN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A generated graph as 0-based sorted CSR (out-lists; in-lists for digraphs).
 * m = edges counted once (undirected) or arcs (directed). */
typedef struct lgbc_csr {
  int64_t n;
  int64_t nnz;
  int64_t m;
  int directed;
  int64_t *rowptr;
  int32_t *colidx;
  int64_t *in_rowptr; /* NULL for undirected graphs */
  int32_t *in_colidx;
} lgbc_csr;

/* R-MAT / Kronecker (randgraphs.jl:1126-1152): 2^scale vertices,
 * edgefactor * 2^scale draws, quadrant probabilities a, b, c (d = 1-a-b-c)
 * chosen bit by bit, vertex ids permuted at random; self-loops and duplicate
 * edges are dropped, and for directed == 0 every edge is stored both ways. */
int lgbc_gen_rmat(int scale, int edgefactor, double a, double b, double c, uint64_t seed,
                  int directed, lgbc_csr *out);

/* Erdos-Renyi G(n, m) as SimpleGraph(nv, ne; seed) / SimpleDiGraph(nv, ne)
 * (randgraphs.jl:25-40, 62-76): uniform (u, v), u != v, rejected when the
 * edge exists, until m edges.  Requires m <= 2/3 of the maximum (the
 * reference takes a complement above that; not needed here). */
int lgbc_gen_erdos_renyi(int64_t n, int64_t m, uint64_t seed, int directed, lgbc_csr *out);

/* barabasi_albert(n, k) (randgraphs.jl:391-392, 449-512): k isolated seed
 * vertices; vertex k+1 links to all of them; each later vertex links to k
 * distinct vertices drawn with probability proportional to degree.  Undirected;
 * m = k * (n - k). */
int lgbc_gen_barabasi_albert(int64_t n, int k, uint64_t seed, lgbc_csr *out);

/* Free the arrays of a generated graph (safe on a zeroed struct). */
void lgbc_csr_free(lgbc_csr *g);

#ifdef __cplusplus
}
#endif

#endif /* LGBC_GEN_H */
