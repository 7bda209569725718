/*
 * CPU restatement of graphops' PageRank / personalized-PageRank power
 * iteration, in FP64, with the reference's loop order and summation order.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: tests, the smoke check
 * and the CPU-baseline leg of bench.py load it to check or time against.  The
 * product path (libgops.so) never links or calls it.
 *
 * Parity is pinned by the reference's own known-answer tests (invariants,
 * doctests, the 4-node example) and by closed forms; the reference crate
 * holds no golden vectors and cannot be built here (it is Rust; no cargo).
 *
 * Graph input is the out-adjacency in ADAPTER order: row u of (row_ptr, col)
 * lists graph.neighbors(u) exactly as the reference's `Graph` adapter returns
 * it (duplicates allowed).  For the weighted variant w[e] is the value of
 * graph.edge_weight(u, col[e]) for that neighbor entry (raw, unclamped).
 *
 * Build: oracle/build_oracle.py (gcc -O2 -ffp-contract=off, so x86 and Arm
 * give bit-identical FP64 results).
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <time.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    double damping;
    uint64_t max_iterations;
    double tolerance;
} orc_config;

typedef struct {
    uint64_t iterations;
    double diff_l1;
    int32_t converged;
} orc_run;

/* Rust's f64::max: if one argument is NaN the other is returned; fmax has the
 * same rule.  Used for `edge_weight(..).max(0.0)` (src/pagerank.rs:231,257). */
static double rust_max(double a, double b) { return fmax(a, b); }

/* Result of the `n == 0` early return (src/pagerank.rs:123-131). */
static void empty_run(orc_run *r) {
    r->iterations = 0;
    r->diff_l1 = 0.0;
    r->converged = 1;
}

/* Sequential L1 residual, old-new (src/pagerank.rs:169-173). */
static double l1_seq(const double *a, const double *b, int64_t n) {
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += fabs(a[i] - b[i]);
    return s;
}

/*
 * pagerank_run, src/pagerank.rs:122-187.
 * scores: caller buffer of n doubles; receives the returned (new) vector.
 */
int orc_pagerank_run(int64_t n, const int64_t *row_ptr, const int32_t *col,
                     orc_config cfg, double *scores, orc_run *run) {
    if (n == 0) { empty_run(run); return 0; }
    const double n_f64 = (double)n;
    double *x = scores;
    double *nx = (double *)malloc(sizeof(double) * (size_t)n);
    if (!nx) return -1;
    for (int64_t i = 0; i < n; ++i) x[i] = 1.0 / n_f64;          /* :133 */
    uint64_t iters = 0;
    double last_diff = INFINITY;
    int converged = 0;
    for (uint64_t it = 0; it < cfg.max_iterations; ++it) {       /* :142 */
        iters += 1;
        double dangling_sum = 0.0;                               /* :144-149 */
        for (int64_t i = 0; i < n; ++i)
            if (row_ptr[i + 1] == row_ptr[i]) dangling_sum += x[i];
        const double dangling_contrib = cfg.damping * dangling_sum / n_f64;
        const double teleport = (1.0 - cfg.damping) / n_f64;
        const double fill = teleport + dangling_contrib;          /* :152 */
        for (int64_t i = 0; i < n; ++i) nx[i] = fill;
        for (int64_t u = 0; u < n; ++u) {                        /* :154-162 */
            const int64_t deg = row_ptr[u + 1] - row_ptr[u];
            if (deg > 0) {
                const double share = cfg.damping * x[u] / (double)deg;
                for (int64_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e)
                    nx[col[e]] += share;
            }
        }
        const double diff = l1_seq(x, nx, n);                    /* :169-173 */
        last_diff = diff;
        double *t = x; x = nx; nx = t;                           /* :175 */
        if (diff < cfg.tolerance) { converged = 1; break; }      /* :176 */
    }
    if (x != scores) { memcpy(scores, x, sizeof(double) * (size_t)n); free(x); }
    else free(nx);
    run->iterations = iters;
    run->diff_l1 = last_diff;
    run->converged = converged;
    return 0;
}

/*
 * pagerank_weighted_run, src/pagerank.rs:210-289.
 * w[e] is edge_weight(u, col[e]) as the adapter returns it; it is clamped with
 * Rust's max(.., 0.0) here, at the two places the reference clamps.
 */
int orc_pagerank_weighted_run(int64_t n, const int64_t *row_ptr,
                              const int32_t *col, const double *w,
                              orc_config cfg, double *scores, orc_run *run) {
    if (n == 0) { empty_run(run); return 0; }
    const double n_f64 = (double)n;
    double *x = scores;
    double *nx = (double *)malloc(sizeof(double) * (size_t)n);
    double *ws = (double *)malloc(sizeof(double) * (size_t)n);
    if (!nx || !ws) { free(nx); free(ws); return -1; }
    for (int64_t i = 0; i < n; ++i) x[i] = 1.0 / n_f64;          /* :222 */
    for (int64_t u = 0; u < n; ++u) {                            /* :227-234 */
        double s = 0.0;
        for (int64_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e)
            s += rust_max(w[e], 0.0);
        ws[u] = s;
    }
    uint64_t iters = 0;
    double last_diff = INFINITY;
    int converged = 0;
    for (uint64_t it = 0; it < cfg.max_iterations; ++it) {
        iters += 1;
        double dangling_sum = 0.0;                               /* :241-246 */
        for (int64_t i = 0; i < n; ++i)
            if (ws[i] == 0.0) dangling_sum += x[i];
        const double dangling_contrib = cfg.damping * dangling_sum / n_f64;
        const double teleport = (1.0 - cfg.damping) / n_f64;
        const double fill = teleport + dangling_contrib;
        for (int64_t i = 0; i < n; ++i) nx[i] = fill;
        for (int64_t u = 0; u < n; ++u) {                        /* :252-263 */
            const double wsu = ws[u];
            if (wsu > 0.0) {
                for (int64_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e) {
                    const double we = rust_max(w[e], 0.0);
                    if (we > 0.0) nx[col[e]] += cfg.damping * x[u] * (we / wsu);
                }
            }
        }
        const double diff = l1_seq(x, nx, n);
        last_diff = diff;
        double *t = x; x = nx; nx = t;
        if (diff < cfg.tolerance) { converged = 1; break; }
    }
    if (x != scores) { memcpy(scores, x, sizeof(double) * (size_t)n); free(x); }
    else free(nx);
    free(ws);
    run->iterations = iters;
    run->diff_l1 = last_diff;
    run->converged = converged;
    return 0;
}

/*
 * personalized_pagerank_run, src/ppr.rs:90-156.  Unweighted; the dangling
 * mass goes back to p (src/ppr.rs:125-128), not uniformly.
 * p: n raw personalization entries (normalised here, src/ppr.rs:104-109).
 */
int orc_ppr_run(int64_t n, const int64_t *row_ptr, const int32_t *col,
                const double *p, orc_config cfg, double *scores, orc_run *run) {
    if (n == 0) { empty_run(run); return 0; }
    double *pv = (double *)malloc(sizeof(double) * (size_t)n);
    double *nx = (double *)malloc(sizeof(double) * (size_t)n);
    if (!pv || !nx) { free(pv); free(nx); return -1; }
    double p_sum = 0.0;
    for (int64_t i = 0; i < n; ++i) p_sum += p[i];
    if (p_sum > 0.0) {
        for (int64_t i = 0; i < n; ++i) pv[i] = p[i] / p_sum;
    } else {
        for (int64_t i = 0; i < n; ++i) pv[i] = 1.0 / (double)n;
    }
    double *x = scores;
    memcpy(x, pv, sizeof(double) * (size_t)n);                   /* :110 */
    uint64_t iters = 0;
    double last_diff = INFINITY;
    int converged = 0;
    for (uint64_t it = 0; it < cfg.max_iterations; ++it) {
        iters += 1;
        double dangling_sum = 0.0;                               /* :119-124 */
        for (int64_t i = 0; i < n; ++i)
            if (row_ptr[i + 1] == row_ptr[i]) dangling_sum += x[i];
        for (int64_t i = 0; i < n; ++i)                          /* :125-128 */
            nx[i] = (1.0 - cfg.damping) * pv[i] +
                    cfg.damping * dangling_sum * pv[i];
        for (int64_t u = 0; u < n; ++u) {                        /* :129-137 */
            const int64_t deg = row_ptr[u + 1] - row_ptr[u];
            if (deg > 0) {
                const double share = cfg.damping * x[u] / (double)deg;
                for (int64_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e)
                    nx[col[e]] += share;
            }
        }
        const double diff = l1_seq(x, nx, n);                    /* :138-142 */
        last_diff = diff;
        double *t = x; x = nx; nx = t;
        if (diff < cfg.tolerance) { converged = 1; break; }      /* :145 */
    }
    if (x != scores) { memcpy(scores, x, sizeof(double) * (size_t)n); free(x); }
    else free(nx);
    free(pv);
    run->iterations = iters;
    run->diff_l1 = last_diff;
    run->converged = converged;
    return 0;
}

/*
 * AdjacencyMatrix::neighbors, src/graph.rs:128-135: {j : M[u][j] > 0.0} in
 * ascending j; the weighted view returns the raw cell (src/graph.rs:139-141).
 * M is row-major n*n.  Writes row_ptr (n+1); col / w (capacity cap, w may be
 * NULL).  Returns the number of edges, or -1 when cap is too small.
 */
int64_t orc_dense_to_csr(int64_t n, const double *M, int64_t *row_ptr,
                         int32_t *col, double *w, int64_t cap) {
    int64_t m = 0;
    row_ptr[0] = 0;
    for (int64_t u = 0; u < n; ++u) {
        const double *row = M + u * n;
        for (int64_t j = 0; j < n; ++j) {
            if (row[j] > 0.0) {
                if (m >= cap) return -1;
                col[m] = (int32_t)j;
                if (w) w[m] = row[j];
                ++m;
            }
        }
        row_ptr[u + 1] = m;
    }
    return m;
}

/*
 * The reference's pagerank_run called with an AdjacencyMatrix: the O(n^2)
 * neighbor precompute (src/pagerank.rs:136, src/graph.rs:128-135) followed by
 * the power iteration.  This is what a caller of the reference pays at the
 * dense 2,000-node configuration, and what the CPU baseline times there.
 */
int orc_pagerank_run_dense(int64_t n, const double *M, orc_config cfg,
                           double *scores, orc_run *run) {
    if (n == 0) { empty_run(run); return 0; }
    int64_t cap = 0;
    for (int64_t i = 0; i < n * n; ++i) cap += (M[i] > 0.0);
    int64_t *rp = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
    int32_t *cl = (int32_t *)malloc(sizeof(int32_t) * (size_t)(cap ? cap : 1));
    if (!rp || !cl) { free(rp); free(cl); return -1; }
    orc_dense_to_csr(n, M, rp, cl, NULL, cap);
    int rc = orc_pagerank_run(n, rp, cl, cfg, scores, run);
    free(rp);
    free(cl);
    return rc;
}

/* ---- many independent PPR solves over host threads (CPU baseline) ---- */

typedef struct {
    int64_t n;
    const int64_t *row_ptr;
    const int32_t *col;
    orc_config cfg;
    const int64_t *seed_ptr;
    const int32_t *seed_idx;
    int64_t first, stride, count;
    double *out;        /* count * n, or NULL */
    uint64_t *iters;    /* count, or NULL */
    int rc;
} ppr_job;

static void *ppr_worker(void *arg) {
    ppr_job *j = (ppr_job *)arg;
    double *p = (double *)calloc((size_t)j->n, sizeof(double));
    double *s = (double *)malloc(sizeof(double) * (size_t)j->n);
    if (!p || !s) { j->rc = -1; free(p); free(s); return NULL; }
    for (int64_t c = j->first; c < j->count; c += j->stride) {
        for (int64_t k = j->seed_ptr[c]; k < j->seed_ptr[c + 1]; ++k)
            p[j->seed_idx[k]] += 1.0;
        orc_run r;
        if (orc_ppr_run(j->n, j->row_ptr, j->col, p, j->cfg, s, &r)) { j->rc = -1; break; }
        if (j->out) memcpy(j->out + c * j->n, s, sizeof(double) * (size_t)j->n);
        if (j->iters) j->iters[c] = r.iterations;
        for (int64_t k = j->seed_ptr[c]; k < j->seed_ptr[c + 1]; ++k)
            p[j->seed_idx[k]] = 0.0;
    }
    free(p);
    free(s);
    return NULL;
}

/*
 * Runs orc_ppr_run once per seed set (personalization = 1 on each seed node),
 * spread round-robin over `threads` host threads.  Each call is the
 * single-threaded reference algorithm; the threads only run independent
 * calls side by side.
 */
int orc_ppr_many(int64_t n, const int64_t *row_ptr, const int32_t *col,
                 orc_config cfg, int64_t nsets, const int64_t *seed_ptr,
                 const int32_t *seed_idx, int threads, double *out,
                 uint64_t *iters) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    ppr_job jobs[256];
    pthread_t tid[256];
    for (int t = 0; t < threads; ++t) {
        jobs[t] = (ppr_job){n, row_ptr, col, cfg, seed_ptr, seed_idx,
                            t, threads, nsets, out, iters, 0};
        if (threads == 1) ppr_worker(&jobs[t]);
        else pthread_create(&tid[t], NULL, ppr_worker, &jobs[t]);
    }
    int rc = 0;
    for (int t = 0; t < threads; ++t) {
        if (threads > 1) pthread_join(tid[t], NULL);
        rc |= jobs[t].rc;
    }
    return rc;
}

/*
 * katz_centrality_run, src/katz.rs:136-201: x = beta; each step
 * new = beta, then for u ascending, for v in neighbors(u): new[v] += alpha*x[u];
 * diff = sequential sum |old - new|; swap; stop when diff < tol.
 * Returns the last new vector; diff_l1 = INFINITY when no step ran.
 */
int orc_katz_run(int64_t n, const int64_t *row_ptr, const int32_t *col, double alpha,
                 double beta, uint64_t max_iterations, double tolerance, double *scores,
                 orc_run *run) {
    if (n == 0) {
        empty_run(run);
        return 0;
    }
    double *x = scores, *y = (double *)malloc(sizeof(double) * (size_t)n);
    if (!y) return 1;
    for (int64_t i = 0; i < n; ++i) x[i] = beta;
    uint64_t iters = 0;
    double last = INFINITY;
    int conv = 0;
    for (uint64_t k = 0; k < max_iterations; ++k) {
        iters += 1;
        for (int64_t i = 0; i < n; ++i) y[i] = beta;
        for (int64_t u = 0; u < n; ++u) {
            const double contrib = alpha * x[u];
            for (int64_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e)
                if (col[e] < n) y[col[e]] += contrib;
        }
        const double diff = l1_seq(x, y, n);
        last = diff;
        double *t = x; x = y; y = t;
        if (diff < tolerance) {
            conv = 1;
            break;
        }
    }
    if (x != scores) {
        memcpy(scores, x, sizeof(double) * (size_t)n);
        y = x;
    }
    free(y);
    run->iterations = iters;
    run->diff_l1 = last;
    run->converged = conv;
    return 0;
}

/*
 * eigenvector_centrality_run, src/eigenvector.rs:49-125: x = 1/sqrt(n);
 * new[v] = x[v] + sum over neighbors(v) of x[u]; L2-normalise with the sign
 * that makes the sum non-negative (skipped when the norm is 0); diff =
 * sequential sum |old - new|; swap; stop when diff < tol.
 */
int orc_eigenvector_run(int64_t n, const int64_t *row_ptr, const int32_t *col,
                        uint64_t max_iterations, double tolerance, double *scores, orc_run *run) {
    if (n == 0) {
        empty_run(run);
        return 0;
    }
    double *x = scores, *y = (double *)malloc(sizeof(double) * (size_t)n);
    if (!y) return 1;
    const double init = 1.0 / sqrt((double)n);
    for (int64_t i = 0; i < n; ++i) x[i] = init;
    uint64_t iters = 0;
    double diff = 0.0;
    int conv = 0;
    for (uint64_t k = 0; k < max_iterations; ++k) {
        iters = k + 1;
        for (int64_t v = 0; v < n; ++v) {
            double s = x[v];
            for (int64_t e = row_ptr[v]; e < row_ptr[v + 1]; ++e)
                if (col[e] < n) s += x[col[e]];
            y[v] = s;
        }
        double sq = 0.0, su = 0.0;
        for (int64_t v = 0; v < n; ++v) sq += y[v] * y[v];
        const double norm = sqrt(sq);
        if (norm > 0.0) {
            for (int64_t v = 0; v < n; ++v) su += y[v];
            const double sign = su >= 0.0 ? 1.0 : -1.0;
            for (int64_t v = 0; v < n; ++v) y[v] = y[v] * sign / norm;
        }
        diff = l1_seq(x, y, n);
        double *t = x; x = y; y = t;
        if (diff < tolerance) {
            conv = 1;
            break;
        }
    }
    if (x != scores) {
        memcpy(scores, x, sizeof(double) * (size_t)n);
        y = x;
    }
    free(y);
    run->iterations = iters;
    run->diff_l1 = diff;
    run->converged = conv;
    return 0;
}

/* l2_normalize and l2_diff, src/centrality.rs:168-183 (sequential sums). */
static void l2n(double *v, int64_t n) {
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += v[i] * v[i];
    const double norm = sqrt(s);
    if (norm > 0.0)
        for (int64_t i = 0; i < n; ++i) v[i] /= norm;
}

static double l2d(const double *a, const double *b, int64_t n) {
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += (a[i] - b[i]) * (a[i] - b[i]);
    return sqrt(s);
}

/*
 * hits, src/centrality.rs:114-166.  The in-neighbour lists are built by
 * scanning u ascending (so each list is in source order, duplicates kept);
 * auth' = l2n(sum over in-neighbours of hub), hub' = l2n(sum over
 * neighbors(u) of auth'); stop when both L2 changes < tol.  run receives the
 * step count, max(auth_diff, hub_diff) of the last step, and convergence.
 */
int orc_hits_run(int64_t n, const int64_t *row_ptr, const int32_t *col, uint64_t max_iterations,
                 double tolerance, double *hub, double *auth, orc_run *run) {
    if (n == 0) {
        empty_run(run);
        return 0;
    }
    const int64_t m = row_ptr[n];
    int64_t *irp = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
    int32_t *icol = (int32_t *)malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1));
    int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    double *na = (double *)malloc(sizeof(double) * (size_t)n);
    double *nh = (double *)malloc(sizeof(double) * (size_t)n);
    if (!irp || !icol || !fill || !na || !nh) {
        free(irp); free(icol); free(fill); free(na); free(nh);
        return 1;
    }
    for (int64_t e = 0; e < m; ++e) irp[col[e] + 1] += 1;
    for (int64_t v = 0; v < n; ++v) irp[v + 1] += irp[v];
    for (int64_t v = 0; v < n; ++v) fill[v] = irp[v];
    for (int64_t u = 0; u < n; ++u)
        for (int64_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e) icol[fill[col[e]]++] = (int32_t)u;
    const double init = 1.0 / sqrt((double)n);
    for (int64_t i = 0; i < n; ++i) hub[i] = auth[i] = init;
    uint64_t iters = 0;
    double last = 0.0;
    int conv = 0;
    for (uint64_t k = 0; k < max_iterations; ++k) {
        iters = k + 1;
        for (int64_t v = 0; v < n; ++v) {
            double s = 0.0;
            for (int64_t e = irp[v]; e < irp[v + 1]; ++e) s += hub[icol[e]];
            na[v] = s;
        }
        l2n(na, n);
        for (int64_t u = 0; u < n; ++u) {
            double s = 0.0;
            for (int64_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e) s += na[col[e]];
            nh[u] = s;
        }
        l2n(nh, n);
        const double ad = l2d(auth, na, n), hd = l2d(hub, nh, n);
        last = ad > hd ? ad : hd;
        memcpy(auth, na, sizeof(double) * (size_t)n);
        memcpy(hub, nh, sizeof(double) * (size_t)n);
        if (ad < tolerance && hd < tolerance) {
            conv = 1;
            break;
        }
    }
    free(irp); free(icol); free(fill); free(na); free(nh);
    run->iterations = iters;
    run->diff_l1 = last;
    run->converged = conv;
    return 0;
}

/*
 * All-cores CPU figure for the weighted PageRank workload (a timing baseline,
 * not a parity reference): the same iteration as pagerank_weighted_run
 * (src/pagerank.rs:210-289: uniform start, dangling <=> weight sum 0, mass
 * spread uniformly, transition max(w,0)/ws, L1 stop with strict <), in pull
 * form over an in-edge CSR so that `threads` host threads each own a range of
 * rows; the sums run in a different order than the reference's scatter.  The
 * in-CSR is built first (not timed); *iter_seconds is the wall time of the
 * iterations alone.
 */
typedef struct {
    int64_t v0, v1;
    const int64_t *irp;
    const int32_t *isrc;
    const double *ip;
    const double *ws;
    double damping, n_f64;
    double **x, **nx;
    double *part_l1, *part_dang;
    int tid;
    pthread_barrier_t *bar;
    uint64_t max_iter;
    double tol;
    int *stop;
    uint64_t *iters;
    double *last_diff;
    int *converged;
    int nthreads;
} pr_mt_job;

static void *pr_mt_worker(void *arg) {
    pr_mt_job *j = (pr_mt_job *)arg;
    for (uint64_t it = 0; it < j->max_iter; ++it) {
        /* dangling mass of x (partials from the previous pass, or initial) */
        double dsum = 0.0;
        for (int t = 0; t < j->nthreads; ++t) dsum += j->part_dang[t];
        const double fill = (1.0 - j->damping) / j->n_f64 + j->damping * dsum / j->n_f64;
        pthread_barrier_wait(j->bar);  /* everyone has read part_dang */
        const double *x = *j->x;
        double *nx = *j->nx;
        double l1 = 0.0, dg = 0.0;
        for (int64_t v = j->v0; v < j->v1; ++v) {
            double s = 0.0;
            for (int64_t e = j->irp[v]; e < j->irp[v + 1]; ++e) s += x[j->isrc[e]] * j->ip[e];
            const double nv = fill + j->damping * s;
            nx[v] = nv;
            l1 += fabs(x[v] - nv);
            if (j->ws[v] == 0.0) dg += nv;
        }
        j->part_l1[j->tid] = l1;
        j->part_dang[j->tid] = dg;
        pthread_barrier_wait(j->bar);
        if (j->tid == 0) {
            double diff = 0.0;
            for (int t = 0; t < j->nthreads; ++t) diff += j->part_l1[t];
            *j->iters = it + 1;
            *j->last_diff = diff;
            double *tmp = *j->x; *j->x = *j->nx; *j->nx = tmp;
            if (diff < j->tol) { *j->converged = 1; *j->stop = 1; }
        }
        pthread_barrier_wait(j->bar);
        if (*j->stop) break;
    }
    return NULL;
}

int orc_pagerank_weighted_run_mt(int64_t n, const int64_t *row_ptr, const int32_t *col, const double *w,
                                 orc_config cfg, int threads, double *scores, orc_run *run,
                                 double *iter_seconds) {
    *iter_seconds = 0.0;
    if (n == 0) { empty_run(run); return 0; }
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    const int64_t m = row_ptr[n];
    double *ws = (double *)calloc((size_t)n, sizeof(double));
    int64_t *irp = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
    int32_t *isrc = (int32_t *)malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1));
    double *ip = (double *)malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
    double *xa = (double *)malloc(sizeof(double) * (size_t)n);
    double *xb = (double *)malloc(sizeof(double) * (size_t)n);
    int64_t *fillp = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    if (!ws || !irp || !isrc || !ip || !xa || !xb || !fillp) {
        free(ws); free(irp); free(isrc); free(ip); free(xa); free(xb); free(fillp);
        return -1;
    }
    for (int64_t u = 0; u < n; ++u) {
        double s = 0.0;
        for (int64_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e) s += rust_max(w[e], 0.0);
        ws[u] = s;
    }
    for (int64_t u = 0; u < n; ++u)
        if (ws[u] > 0.0)
            for (int64_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e)
                if (rust_max(w[e], 0.0) > 0.0) irp[col[e] + 1] += 1;
    for (int64_t v = 0; v < n; ++v) irp[v + 1] += irp[v];
    memcpy(fillp, irp, sizeof(int64_t) * (size_t)n);
    for (int64_t u = 0; u < n; ++u)
        if (ws[u] > 0.0)
            for (int64_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e) {
                const double we = rust_max(w[e], 0.0);
                if (we > 0.0) {
                    const int64_t q = fillp[col[e]]++;
                    isrc[q] = (int32_t)u;
                    ip[q] = we / ws[u];
                }
            }
    free(fillp);
    for (int64_t i = 0; i < n; ++i) xa[i] = 1.0 / (double)n;
    double part_l1[256], part_dang[256];
    for (int t = 0; t < threads; ++t) { part_l1[t] = 0.0; part_dang[t] = 0.0; }
    double d0 = 0.0;
    for (int64_t i = 0; i < n; ++i)
        if (ws[i] == 0.0) d0 += xa[i];
    part_dang[0] = d0;
    double *xp = xa, *nxp = xb;
    int stop = 0, converged = 0;
    uint64_t iters = 0;
    double last_diff = INFINITY;
    pthread_barrier_t bar;
    pthread_barrier_init(&bar, NULL, (unsigned)threads);
    pr_mt_job jobs[256];
    pthread_t tid[256];
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int t = 0; t < threads; ++t) {
        jobs[t] = (pr_mt_job){n * t / threads, n * (t + 1) / threads, irp, isrc, ip, ws, cfg.damping,
                              (double)n, &xp, &nxp, part_l1, part_dang, t, &bar, cfg.max_iterations,
                              cfg.tolerance, &stop, &iters, &last_diff, &converged, threads};
        if (t > 0) pthread_create(&tid[t], NULL, pr_mt_worker, &jobs[t]);
    }
    pr_mt_worker(&jobs[0]);
    for (int t = 1; t < threads; ++t) pthread_join(tid[t], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    *iter_seconds = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
    pthread_barrier_destroy(&bar);
    memcpy(scores, xp, sizeof(double) * (size_t)n);
    free(ws); free(irp); free(isrc); free(ip); free(xa); free(xb);
    run->iterations = iters;
    run->diff_l1 = last_diff;
    run->converged = converged;
    return 0;
}
