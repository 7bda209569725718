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
 *  - Device memory is owned by gops_ctx / gops_graph / gops_warm objects and
 *    released by their destroy functions, which may run in any order (a
 *    graph or model may outlive the context that created it, for destruction
 *    only).
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
/* Test hook (no reference counterpart): host-side fault injection.  With
 * count >= 0 the next `count` device allocations of the library's pool
 * succeed and every later one fails as if the device were out of memory
 * (GOPS_ERR_OOM from the call that needed it), until called with count < 0.
 * Lets tests drive every allocation-failure path without a GPU fault. */
int gops_debug_fail_allocations_after(int64_t count);
/* Test hook (no reference counterpart): one call of the warm start's
 * tensor-core row-tile GEMM (tcgen05, TMA-fed) on caller device buffers, all
 * BF16 row-major but bias/head/w (FP32).  Synchronous.
 *   mode 0 (layer 2): out[m][128] = relu([xa | xb] bt^T + bias) with xa, xb
 *     m x 128 and bt 128 x 256; w[i] = exp(clamp(out[i] . head[0:128] +
 *     head[128], -20, 20)) from the rounded out row.
 *   mode 1 (input gradient): out[m][256] = xa bt^T, xa m x 128, bt 256 x 128;
 *     xb, bias, head and w are not used.
 * err: a device int, set nonzero when a handshake wait in the kernel ran out
 * (the kernel then winds down instead of hanging). */
int gops_debug_tc_gemm(gops_ctx *ctx, int mode, const void *xa, const void *xb, const void *bt, int64_t m, void *out,
                       const float *bias, const float *head, float *w, int *err);
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
 * Requires n < 2^31 - 1 and m < 2^31 - 1 (int32 indices on the device). */
int gops_graph_upload(gops_ctx *ctx, int64_t n, const int64_t *row_ptr, const int32_t *col,
                      const double *weights, gops_graph **out);

/* AdjacencyMatrix (src/graph.rs:122-142): a row-major n*n f64 matrix; edge
 * u->j iff M[u][j] > 0.0, weight M[u][j].  The O(n^2) scan runs on the
 * device. */
int gops_graph_from_dense(gops_ctx *ctx, int64_t n, const double *matrix, gops_graph **out);

/* The petgraph adapters in bulk (src/graph.rs:144-212, feature petgraph):
 * instead of calling neighbors(u) and find_edge per node (one Vec per node,
 * src/graph.rs:163-197), a Rust caller passes the raw edge list of its
 * petgraph::Graph<_, f64, Directed> as stored (edge e: src[e] -> dst[e],
 * weights[e] optional; graph.raw_edges() in edge-index order), and the device
 * builds the out-adjacency the adapter exposes: row u lists the targets of
 * u's outgoing edges newest first (petgraph's neighbors order; parallel
 * edges repeated), and with weights every u -> v entry carries the weight
 * find_edge(u, v) returns, the newest u -> v edge's.  Then as
 * gops_graph_upload.  n, m < 2^31 - 1; an endpoint outside [0, n) is
 * refused. */
int gops_graph_from_edges(gops_ctx *ctx, int64_t n, int64_t m, const int32_t *src, const int32_t *dst,
                          const double *weights, gops_graph **out);

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
 * calls (src/ppr.rs:90-156) in one pass per wave of 32, 64 or 128 sets (the
 * k-tile, chosen per graph by an autotuner on the first call; see
 * gops_ppr_batch_set_tile).  Set s is
 * seed_idx[seed_ptr[s] .. seed_ptr[s+1]) (node ids; a repeated node counts
 * twice); its personalization vector is 1 on each seed, normalised as
 * src/ppr.rs:104-109 does, and an empty set means the uniform vector.  Each
 * set stops at its own first step whose L1 norm is below tolerance.
 * x0 (optional, nsets*n floats, set-major, original node order) replaces the
 * start vector p by a caller-supplied one (a warm start, such as the learned
 * one); the iteration and its stopping rule are unchanged.
 * scores (optional): nsets*n floats, set-major, original node order (FP32);
 * page-locked host memory (cudaHostAlloc, cudaHostRegister) is written by
 * DMA from each wave's block while the next wave runs, other host memory
 * through the context's pinned staging buffers and a host copy.
 * runs (optional): nsets run records. */
int gops_ppr_batch(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg, int64_t nsets,
                   const int64_t *seed_ptr, const int32_t *seed_idx, const float *x0,
                   float *scores, gops_run *runs);

/* As gops_ppr_batch, with x0 and scores in device memory (CUDA pointers,
 * e.g. from another framework): no host copies of the score blocks. */
int gops_ppr_batch_device(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg, int64_t nsets,
                          const int64_t *seed_ptr, const int32_t *seed_idx, const float *x0_device,
                          float *scores_device, gops_run *runs);

/* The batched path's tile of a graph: cols = sets per wave (32, 64 or 128),
 * chunk = the in-degree above which a row is split into chunks of that many
 * edges (a multiple of 256), l2_hints = the FP32 step marks the hottest rows
 * of the gathered block evict-last in L2 and its streams evict-first.
 * cols == 0 re-runs the autotuner, which times a few steps of each k-tile x
 * chunk 256 / 1024 (within 40 % of the free device memory), keeps the
 * fastest per set-step, then times that tile with L2 hints.  The tile
 * changes the time only: every choice gives bit-identical results (a row's
 * sum is fixed as in-order sums of 256-edge blocks added in order, and each
 * set's precision phases depend on its own step norms only).  No reference
 * counterpart (the reference solves one set per call). */
int gops_ppr_batch_set_tile(gops_ctx *ctx, const gops_graph *g, int32_t cols, int32_t chunk, int32_t l2_hints);
/* The tile in use (0, 0, 0 before the first batched call), and with
 * cost != NULL the autotuner's measured cost per set-step in ms: 7 floats,
 * (cols 32, 64, 128) x (chunk 256, 1024) without L2 hints, then the chosen
 * tile with them; 0 where not tried. */
int gops_ppr_batch_tile(const gops_graph *g, int32_t *cols, int32_t *chunk, int32_t *l2_hints, float *cost);

/* Device pointer (double, n entries) of the last solve's scores, valid until
 * the next solve on this context or the destruction of the graph that solve
 * ran on, whichever comes first (the vector lives in the graph's workspace).
 * After gops_pagerank_run_noalloc the vector lives in that entry point's
 * shared scratch array instead: it is valid only until the next no-alloc
 * call on the same device, from any context. */
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
 * The array is mapped on a device when the first context on it is created
 * (gops_ctx_create loads its module and looks up its address, so that no
 * later call needs device memory for it, also under CUDA's lazy module
 * loading); the address is dropped with the device's last context.  After
 * a call, gops_ctx_scores_device points into the shared array. */
int gops_pagerank_run_noalloc(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg,
                              double *scores, gops_run *run);

/* ---- Katz and eigenvector centrality: the same pull power iteration ---- */

/* KatzConfig (src/katz.rs:19-57): attenuation alpha, baseline beta,
 * max_iterations, tolerance on the L1 norm of the step. */
typedef struct gops_katz_config {
  double alpha;
  double beta;
  uint64_t max_iterations;
  double tolerance;
} gops_katz_config;

/* KatzConfig::validate (src/katz.rs:60-86): the reference's messages. */
int gops_katz_config_validate(const gops_katz_config *cfg, char *msg, size_t msg_cap);

/* katz_centrality_run (src/katz.rs:136-201): x_0 = beta, x_{k+1}[v] = beta +
 * alpha * sum over edges u->v of x_k[u] (multi-edges counted, weights
 * ignored), stop at the first step whose L1 norm < tolerance.  FP64.
 * scores: n doubles (or NULL). */
int gops_katz_run(gops_ctx *ctx, const gops_graph *g, const gops_katz_config *cfg, double *scores,
                  gops_run *run);

/* eigenvector_centrality_run (src/eigenvector.rs:49-125): x_0 = 1/sqrt(n),
 * y[v] = x[v] + sum over the out-neighbours u of v of x[u], then y divided by
 * its L2 norm with the sign making its sum non-negative (unchanged when the
 * norm is 0); stop at the first step whose L1 change < tolerance.  FP64. */
int gops_eigenvector_run(gops_ctx *ctx, const gops_graph *g, uint64_t max_iterations, double tolerance,
                         double *scores, gops_run *run);

/* hits (src/centrality.rs:114-166): hub = auth = 1/sqrt(n); each step
 * auth'[v] = sum over edges u->v of hub[u], L2-normalised; hub'[u] = sum over
 * edges u->v of auth'[v], L2-normalised (a zero vector stays as is); stop
 * when both L2 changes are below tolerance.  hub, auth: n doubles each (or
 * NULL).  The reference returns only (hub, auth); run adds the step count,
 * the larger L2 change of the last step and whether both fell below tol.
 * FP64. */
int gops_hits_run(gops_ctx *ctx, const gops_graph *g, uint64_t max_iterations, double tolerance, double *hub,
                  double *auth, gops_run *run);

/* ---- top_k and normalize (src/topk.rs:17-61) on device-resident scores ----
 * The k largest finite, positive scores by score descending (the reference
 * skips non-finite and non-positive entries); equal scores are ordered by
 * index (the reference leaves their order unspecified and keeps, at the
 * boundary, the entries met first: the same set).  k <= 1024.  idx / val:
 * host buffers of k (per row: rows*k) entries; count(s): entries written. */
int gops_top_k_f64_device(gops_ctx *ctx, const double *scores_device, int64_t n, int64_t k, int64_t *idx,
                          double *val, int64_t *count);
/* The same for each row of a row-major FP32 block (rows x n), e.g. the
 * scores of gops_ppr_batch_device: top-k per seed set without copying the
 * block to the host. */
int gops_top_k_f32_rows_device(gops_ctx *ctx, const float *block_device, int64_t rows, int64_t n, int64_t k,
                               int64_t *idx, float *val, int64_t *counts);
/* normalize (src/topk.rs:53-61): divide by the sum when the sum is > 0. */
int gops_normalize_f64_device(gops_ctx *ctx, double *scores_device, int64_t n);

/* ---- learned warm start for batched personalized PageRank ----
 * No counterpart in the reference (it is the extension that feeds
 * gops_ppr_batch's x0).  A per-graph model predicts each set's PPR vector:
 *
 *   x0 = (1-d) (s + d P s + d^2 P^2 s + d^3 P^3 s)          exact, sparse push
 *      + tail_i = tm * w_i * m[a_i] / (sum_c m[c] * cw[a_i])  learned
 *
 * where s is the set's normalised indicator, P the transition matrix,
 * tm = 1 - sum of the exact part, a_i a k-means cluster of node i over a
 * seeded random-projection code (diffusion of Gaussian vectors over the
 * graph), w_i = exp(MPNN(features of i)) a per-node weight from a two-layer
 * message-passing network (hidden 128, BF16 operands, FP32 accumulation) fed
 * log(1+out-degree), log(1+in-degree) and the code, m = relu(c K) the
 * predicted cluster masses from the cluster mix c of P^3 s and P^4 s, and
 * cw[c] = sum of w over cluster c.  K is fitted by least squares and the MPNN
 * by Adam on an L1 loss, both against PPR vectors that gops_ppr_batch
 * computes on the device.  The power iteration still runs to the same
 * tolerance; a warm start whose first residual is not below the cold start's
 * is rejected and the set is solved again from s. */
typedef struct gops_warm gops_warm;

typedef struct gops_warm_config {
  int32_t clusters;     /* k-means clusters, 1..256 (default 128; best kept of 8 seeded runs) */
  int32_t code_steps;   /* diffusion steps of the 16-wide code (default 10) */
  int32_t kmeans_iters; /* Lloyd iterations after k-means++ seeding (default 20) */
  int32_t minibatch;    /* sets per Adam step, 1..32 (default 32) */
  int32_t chunk;        /* training targets solved per batched call (default 512) */
  int32_t epochs;       /* passes over the training sets (default 1) */
  float lr;             /* Adam step size (default 3e-3) */
  float ridge;          /* least-squares ridge, relative to the Gram trace (default 1e-9) */
  uint64_t seed;        /* seeds the code, k-means++ and the initial weights */
  int64_t push_budget;  /* edge visits of one set's push before it starts cold (default 1<<24) */
} gops_warm_config;

typedef struct gops_warm_stats {
  double loss_first;    /* mean L1 loss of the first and last Adam steps */
  double loss_last;
  int64_t steps;        /* Adam steps taken */
  int64_t sets;         /* training targets solved */
  double target_ms;     /* device time: solving the targets */
  double fit_ms;        /* device time: push, least squares and Adam steps */
} gops_warm_stats;

void gops_warm_config_default(gops_warm_config *cfg);

/* Builds the model's graph-side state (CSR copies in original order, code,
 * features, clusters; untrained weights).  row_ptr/col: the out-adjacency
 * given to gops_graph_upload for g. */
int gops_warm_create(gops_ctx *ctx, const gops_graph *g, const int64_t *row_ptr, const int32_t *col,
                     const gops_warm_config *wcfg, gops_warm **out);
void gops_warm_destroy(gops_warm *w);

/* Trains on the given seed sets (layout as gops_ppr_batch): solves their PPR
 * vectors with cfg on the device, fits K and runs the Adam steps. */
int gops_warm_train(gops_ctx *ctx, gops_warm *w, const gops_config *cfg, int64_t nsets,
                    const int64_t *seed_ptr, const int32_t *seed_idx, gops_warm_stats *stats);

/* Warm starts for nsets sets into x0_device (nsets*n floats, set-major,
 * original order).  r1_cold (optional, host, nsets): the first-step residual
 * L1 norm of the cold start of each set.  A set whose push would exceed the
 * budget gets x0 = s and r1_cold = +inf. */
int gops_warm_predict(gops_ctx *ctx, gops_warm *w, double damping, int64_t nsets, const int64_t *seed_ptr,
                      const int32_t *seed_idx, float *x0_device, double *r1_cold);

/* gops_ppr_batch with learned warm starts: predict, solve, and solve again
 * from s every set whose warm start was rejected (rejected: optional host
 * flags, nsets).  scores: host buffer as in gops_ppr_batch, or NULL. */
int gops_ppr_batch_learned(gops_ctx *ctx, const gops_graph *g, gops_warm *w, const gops_config *cfg,
                           int64_t nsets, const int64_t *seed_ptr, const int32_t *seed_idx, float *scores,
                           gops_run *runs, int32_t *rejected);
/* The same with scores in device memory (nsets*n floats). */
int gops_ppr_batch_learned_device(gops_ctx *ctx, const gops_graph *g, gops_warm *w, const gops_config *cfg,
                                  int64_t nsets, const int64_t *seed_ptr, const int32_t *seed_idx,
                                  float *scores_device, gops_run *runs, int32_t *rejected);

/* Batched PPR from caller-supplied warm starts, judged: x0_device (nsets*n
 * floats, set-major) as in gops_ppr_batch_device; a set whose first-step
 * residual L1 norm is not below r1_max[s] (host, optional: NULL accepts every
 * start) is retired after that step and solved again from its
 * personalization vector (rejected[s] = 1).  gops_ppr_batch_learned is
 * gops_warm_predict followed by this call with r1_max = the cold residuals.
 * A set with a finite r1_max[s] leaves the double-float phase at a step norm
 * of 0.5 instead of 0.1 (its first residual is already small); every other
 * set, here or in gops_ppr_batch, keeps 0.1. */
int gops_ppr_batch_judged_device(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg, int64_t nsets,
                                 const int64_t *seed_ptr, const int32_t *seed_idx, const float *x0_device,
                                 const double *r1_max, float *scores_device, gops_run *runs, int32_t *rejected);

/* Model state in and out (host buffers), for checkpoints and for checking the
 * kernels against a CPU restatement.  `what`:
 *   GOPS_WARM_PARAMS   float, gops_warm_param_count() entries (W1 48x128 with
 *                      the layer-1 bias as row 36, W2 256x128, b2 128, w3 128, b3 1)
 *   GOPS_WARM_COUPLING float, (2*clusters+1) x clusters (K)
 *   GOPS_WARM_CLUSTERS int32, n (cluster of each node)
 *   GOPS_WARM_FEATURES float, n x 48 (layer-1 input [x, mean_in x, 1, 0...], as BF16 values)
 *   GOPS_WARM_CODE     float, n x 16
 *   GOPS_WARM_WEIGHT   float, n (w of the current parameters) */
enum {
  GOPS_WARM_PARAMS = 0,
  GOPS_WARM_COUPLING = 1,
  GOPS_WARM_CLUSTERS = 2,
  GOPS_WARM_FEATURES = 3,
  GOPS_WARM_CODE = 4,
  GOPS_WARM_WEIGHT = 5
};
int64_t gops_warm_count(const gops_warm *w, int what);
int gops_warm_get(gops_ctx *ctx, gops_warm *w, int what, void *host, int64_t count);
/* GOPS_WARM_PARAMS and GOPS_WARM_COUPLING only (resets the Adam moments). */
int gops_warm_set(gops_ctx *ctx, gops_warm *w, int what, const void *host, int64_t count);

/* One loss/gradient evaluation without a parameter update: targets_x (host,
 * nsets*n floats, set-major) are the sets' PPR vectors; loss = mean over sets
 * of the L1 error of the predicted tail; grad (host, param count floats) its
 * gradient with respect to GOPS_WARM_PARAMS.  nsets <= 32. */
int gops_warm_loss_grad(gops_ctx *ctx, gops_warm *w, double damping, int64_t nsets, const int64_t *seed_ptr,
                        const int32_t *seed_idx, const float *targets_x, double *loss, float *grad);

/* The exact part of the warm start for one set (host outputs): local (n
 * doubles, the four push terms), mix (2*clusters+1 doubles: cluster mix of
 * P^3 s, of P^4 s, and 1), tail mass and cold first residual.  Returns
 * GOPS_ERR_INVALID when the set exceeds the push budget. */
int gops_warm_push(gops_ctx *ctx, gops_warm *w, double damping, const int32_t *seeds, int64_t nseeds,
                   double *local, double *mix, double *tail_mass, double *r1_cold);

#ifdef __cplusplus
}
#endif
#endif /* GOPS_H */
