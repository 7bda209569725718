/*
 * Seeded synthetic graph generators for the PageRank / PPR workloads.
 *
 * These build the inputs the benchmarks and tests run on (no dataset is
 * read): directed Erdos-Renyi, R-MAT, a stochastic block model, and seed-set
 * samplers.  Output is an out-adjacency CSR (row_ptr int64[n+1], col
 * int32[m], rows ascending, columns ascending within a row) plus optional FP32
 * weights.  All randomness is counter based (SplitMix64 finaliser over
 * (seed, index)), integer thresholds decide every Bernoulli draw, and the
 * library is built with -ffp-contract=off, so a given seed yields the same
 * graph on x86-64 and AArch64 and for any thread count.
 *
 * There is no counterpart in graphops: the reference takes user graphs only.
 */
#ifndef GRAPHGEN_H
#define GRAPHGEN_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gg_graph gg_graph;

/* Directed G(n, p) without self loops; then round(n * dangling_frac) nodes,
 * chosen by a seeded shuffle, lose all their out-edges.  Unit weights. */
gg_graph *gg_erdos_renyi(int64_t n, double p, double dangling_frac, uint64_t seed);

/* R-MAT: edge_factor * 2^scale draws with quadrant probabilities a/b/c/d
 * (d = 1-a-b-c), self loops and duplicates removed.  When `weighted`, each
 * kept edge (u, v) gets w = float(wlo + (whi - wlo) * U(u, v)) with U uniform
 * in [0,1) from a hash of (seed, u, v). */
gg_graph *gg_rmat(int scale, int edge_factor, double a, double b, double c,
                  int weighted, double wlo, double whi, uint64_t seed, int threads);

/* Stochastic block model: `blocks` blocks with sizes proportional to
 * (i+1)^-zipf_s, every node draws Binomial(64, intra/64) targets uniform in
 * its own block (self excluded) and Binomial(64, inter/64) targets uniform
 * outside it; duplicates removed; node ids are then relabelled by a seeded
 * permutation.  block_of (optional, n entries) receives each node's block. */
gg_graph *gg_sbm(int64_t n, int blocks, double zipf_s, double intra_mean,
                 double inter_mean, uint64_t seed, int threads);

int64_t gg_n(const gg_graph *g);
int64_t gg_m(const gg_graph *g);
int gg_weighted(const gg_graph *g);
/* Copies the CSR out; w may be NULL; block_of may be NULL (SBM only). */
void gg_export(const gg_graph *g, int64_t *row_ptr, int32_t *col, float *w,
               int32_t *block_of);
void gg_free(gg_graph *g);

/* Seed sets: nsets sets with sizes uniform in [lo, hi] (clamped to n),
 * distinct nodes within a set, each node drawn with probability proportional
 * to its out-degree (uniform when the graph has no edges).  seed_ptr has
 * nsets+1 entries; seed_idx must hold nsets*hi entries.  Returns total count. */
int64_t gg_seed_sets(int64_t n, const int64_t *row_ptr, int64_t nsets, int lo,
                     int hi, uint64_t seed, int64_t *seed_ptr, int32_t *seed_idx);

/* The SplitMix64 finaliser the generators use (exported for tests). */
uint64_t gg_mix64(uint64_t x);

#ifdef __cplusplus
}
#endif
#endif
