/*
 * libgops: GB300 (sm_103a) PageRank / personalized-PageRank power iteration
 * behind a plain C ABI.
 *
 * This is the drop-in boundary for graphops' PageRank path (crate graphops
 * 0.4.1).  Each entry point names the reference item it stands in for; the
 * Rust API above it (pagerank, pagerank_run, pagerank_weighted,
 * personalized_pagerank, PageRankConfig, the Graph adapters) keeps its
 * signatures and calls these functions through `extern "C"`.
 *
 * Conventions
 *  - Every function returns a gops status (GOPS_OK == 0).  On failure the
 *    context keeps a message, read with gops_last_error().
 *  - All host buffers are owned by the caller; the library copies inputs in
 *    and writes results into caller-allocated outputs.  No pointer passed in
 *    is retained after the call returns.
 *  - Device memory is owned by gops_ctx / gops_graph objects and released by
 *    their destroy functions.
 *  - A context is used by one host thread at a time (one context per thread,
 *    or external locking).  Different contexts may run concurrently.
 *  - Results are deterministic: the same inputs and configuration give
 *    bit-identical outputs on the same GPU model.
 */
#ifndef GOPS_H
#define GOPS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GOPS_ABI_VERSION 1

/* status codes */
#define GOPS_OK 0
#define GOPS_ERR_INVALID 1   /* bad argument (message says which)          */
#define GOPS_ERR_OOM 2       /* device or pinned host allocation failed     */
#define GOPS_ERR_CUDA 3      /* CUDA runtime error                          */
#define GOPS_ERR_TIMEOUT 4   /* a bounded device-side wait ran out          */
#define GOPS_ERR_NO_DEVICE 5 /* no usable CUDA device                       */
#define GOPS_ERR_INTERNAL 6  /* library invariant violated                  */

typedef struct gops_ctx gops_ctx;
typedef struct gops_graph gops_graph;

/* PageRankConfig (src/pagerank.rs:39-49): damping, max_iterations (usize),
 * tolerance on the L1 norm of the step between consecutive iterates. */
typedef struct gops_config {
  double damping;
  uint64_t max_iterations;
  double tolerance;
} gops_config;

/* PageRankRun without its score vector (src/pagerank.rs:16-29); the scores go
 * to the caller's buffer. */
typedef struct gops_run {
  uint64_t iterations; /* update steps performed (== max when not converged) */
  double diff_l1;      /* L1 norm of the last step                           */
  int32_t converged;   /* diff_l1 < tolerance before max_iterations          */
  int32_t reserved;
} gops_run;

/* Per-context counters of the most recent solve (for measurement). */
typedef struct gops_stats {
  double solve_ms;          /* device time of the solve, CUDA events on the ctx stream */
  double iterate_ms;        /* device time spent in the iteration kernels             */
  uint64_t kernel_launches; /* kernels this library launched for the solve            */
  uint64_t iterations;      /* iterations of the solve (sum over columns for batches) */
  uint64_t h2d_bytes;       /* host-to-device bytes copied by the call                */
  uint64_t d2h_bytes;       /* device-to-host bytes copied by the call                */
  /* with gops_ctx_set_timing(ctx, 1): summed CUDA-event durations of the
   * iteration-kernel launches that performed a step, per precision phase */
  double df_ms;
  uint64_t df_launches;
  double f32_ms;
  uint64_t f32_launches;
} gops_stats;

/* ---- library / context (no reference counterpart: the reference is a pure
 * CPU crate with no device state) ---- */
int gops_abi_version(void);
int gops_ctx_create(int device, gops_ctx **out);
void gops_ctx_destroy(gops_ctx *ctx);
const char *gops_last_error(const gops_ctx *ctx);
int gops_ctx_stats(const gops_ctx *ctx, gops_stats *out);
/* The context's CUDA stream (a cudaStream_t), for callers that order their
 * own work against the library's. */
void *gops_ctx_stream(gops_ctx *ctx);
/* Enables (1) or disables (0) per-launch CUDA-event timing of the iteration
 * kernels; the results appear in gops_stats.  Off by default. */
int gops_ctx_set_timing(gops_ctx *ctx, int enable);

/* PageRankConfig::validate (src/pagerank.rs:63-85).  Writes the reference's
 * exact message ("damping must be finite", ...) into msg on failure and
 * returns GOPS_ERR_INVALID. */
int gops_config_validate(const gops_config *cfg, char *msg, size_t msg_cap);

/* Weight checks of pagerank_weighted_checked (src/pagerank.rs:294-316):
 * "edge weights must be finite" / "edge weights must be non-negative". */
int gops_weights_validate(int64_t m, const double *weights, char *msg, size_t msg_cap);

/* Personalization checks of personalized_pagerank_checked (src/ppr.rs:11-44):
 * length, finite, non-negative, sum > 0, with the reference's messages. */
int gops_personalization_validate(int64_t node_count, int64_t len, const double *p,
                                  char *msg, size_t msg_cap);

/* ---- graphs: the Graph / WeightedGraph adapters (src/graph.rs:26-72) ----
 *
 * gops_graph_upload takes the out-adjacency a Graph adapter exposes:
 * row u of (row_ptr[n+1], col[m]) is graph.neighbors(u) in adapter order
 * (duplicates allowed, each counted, as the reference counts them), and
 * weights[e] (optional) is graph.edge_weight(u, col[e]) for that entry.  The
 * device builds the in-edge CSR from it (transpose by stable radix sort),
 * the FP32 transition weights max(w,0)/sum_u max(w,0), and the dangling sets
 * of both the unweighted (deg == 0) and weighted (weight sum == 0) chains.
 * Requires n < 2^31 and m < 2^31. */
int gops_graph_upload(gops_ctx *ctx, int64_t n, const int64_t *row_ptr, const int32_t *col,
                      const double *weights, gops_graph **out);

/* AdjacencyMatrix (src/graph.rs:122-142): a row-major n*n f64 matrix; edge
 * u->j iff M[u][j] > 0.0, weight M[u][j].  The O(n^2) scan runs on the
 * device. */
int gops_graph_from_dense(gops_ctx *ctx, int64_t n, const double *matrix, gops_graph **out);

void gops_graph_destroy(gops_graph *g);
int gops_graph_info(const gops_graph *g, int64_t *n, int64_t *m, int32_t *weighted);

/* ---- the power iterations ----
 * scores: caller buffer of n doubles, or NULL to leave the result on the
 * device (read it with gops_ctx_scores_device). */

/* pagerank_run (src/pagerank.rs:122-187): unweighted, uniform start,
 * dangling mass spread uniformly, stop when the step's L1 norm < tolerance. */
int gops_pagerank_run(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg,
                      double *scores, gops_run *run);

/* pagerank_weighted_run (src/pagerank.rs:210-289): transition
 * max(w,0)/sum max(w,0); a node whose weight sum is 0 is dangling. */
int gops_pagerank_weighted_run(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg,
                               double *scores, gops_run *run);

/* personalized_pagerank_run (src/ppr.rs:90-156): p (n entries) is normalised
 * by its sum, or replaced by uniform when the sum is <= 0; start at p;
 * dangling mass returns to p.  Unweighted. */
int gops_personalized_pagerank_run(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg,
                                   const double *personalization, double *scores, gops_run *run);

/* Batched personalized PageRank: nsets independent personalized_pagerank_run
 * calls (src/ppr.rs:90-156) in one pass per wave of 32 sets.  Set s is
 * seed_idx[seed_ptr[s] .. seed_ptr[s+1]) (node ids; a repeated node counts
 * twice); its personalization vector is 1 on each seed, normalised as
 * src/ppr.rs:104-109 does, and an empty set means the uniform vector.  Each
 * set stops at its own first step whose L1 norm is below tolerance.
 * x0 (optional, nsets*n floats, set-major, original node order) replaces the
 * start vector p by a caller-supplied one (a warm start, such as the learned
 * one); the iteration and its stopping rule are unchanged.
 * scores (optional): nsets*n floats, set-major, original node order (FP32).
 * runs (optional): nsets run records. */
int gops_ppr_batch(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg, int64_t nsets,
                   const int64_t *seed_ptr, const int32_t *seed_idx, const float *x0,
                   float *scores, gops_run *runs);

/* As gops_ppr_batch, with x0 and scores in device memory (CUDA pointers,
 * e.g. from another framework): no host copies of the score blocks. */
int gops_ppr_batch_device(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg, int64_t nsets,
                          const int64_t *seed_ptr, const int32_t *seed_idx, const float *x0_device,
                          float *scores_device, gops_run *runs);

/* Device pointer (double, n entries) of the last solve's scores, valid until
 * the next solve on this context. */
const double *gops_ctx_scores_device(const gops_ctx *ctx);

/* gops_pagerank_run without any allocation.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory when
 * they solve -- a process whose device memory belongs to another allocator
 * (a framework's caching pool), or a latency-critical path where
 * cudaMalloc/cudaFree would synchronize the device.  Same kernels and results
 * as gops_pagerank_run; the per-solve scratch lives in a fixed __device__
 * array of the library (about 13 MB, held by every GPU that loads the
 * library until exit) instead of the graph's workspace.  Limits: at most
 * 262,144 nodes and 65,536 hub tasks, else GOPS_ERR_INVALID.  The graph must
 * already be uploaded (that call allocates).  All calls share the array:
 * calls that overlap on the GPU race and must be serialized by the caller.
 * The first call on a device looks up the array's address, so make it
 * before any stream capture. */
int gops_pagerank_run_noalloc(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg,
                              double *scores, gops_run *run);

#ifdef __cplusplus
}
#endif
#endif /* GOPS_H */
