/*
 * Seeded synthetic graph generators (see graphgen.h for the contract).
 * Built with -O2 -ffp-contract=off -pthread; no architecture-specific code.
 */
#include "graphgen.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

struct gg_graph {
    int64_t n, m;
    int64_t *row_ptr;
    int32_t *col;
    float *w;
    int32_t *block;
};

/* SplitMix64 finaliser (Steele, Lea, Flood 2014). */
uint64_t gg_mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

/* Independent stream `s` of the generator seeded with `seed`, element i. */
static inline uint64_t rnd(uint64_t seed, uint64_t s, uint64_t i) {
    return gg_mix64(gg_mix64(seed ^ (s * 0xd1b54a32d192ed03ULL)) + i * 0x9e3779b97f4a7c15ULL);
}

/* p in [0,1] as a 64-bit threshold: Bernoulli(p) <=> r < thr. */
static uint64_t thr64(double p) {
    if (p <= 0.0) return 0;
    if (p >= 1.0) return UINT64_MAX;
    return (uint64_t)(p * 18446744073709551616.0);
}

static uint32_t thr32(double p) {
    if (p <= 0.0) return 0;
    if (p >= 1.0) return UINT32_MAX;
    return (uint32_t)(p * 4294967296.0);
}

/* ---------------- tiny parallel-for over pthreads ---------------- */

typedef void (*pf_fn)(void *ctx, int tid, int nthreads);
typedef struct { pf_fn fn; void *ctx; int tid, nt; } pf_arg;

static void *pf_tramp(void *a) {
    pf_arg *p = (pf_arg *)a;
    p->fn(p->ctx, p->tid, p->nt);
    return NULL;
}

static void parallel_for(int nt, pf_fn fn, void *ctx) {
    if (nt < 1) nt = 1;
    if (nt > 256) nt = 256;
    if (nt == 1) { fn(ctx, 0, 1); return; }
    pthread_t th[256];
    pf_arg args[256];
    for (int t = 0; t < nt; ++t) {
        args[t] = (pf_arg){fn, ctx, t, nt};
        pthread_create(&th[t], NULL, pf_tramp, &args[t]);
    }
    for (int t = 0; t < nt; ++t) pthread_join(th[t], NULL);
}

static void range_of(int64_t total, int tid, int nt, int64_t *lo, int64_t *hi) {
    *lo = total * tid / nt;
    *hi = total * (tid + 1) / nt;
}

/* ---------------- edge list -> sorted, deduplicated CSR ---------------- */

typedef struct {
    int64_t n, E;
    const uint32_t *src, *dst;
    int64_t *cnt;      /* n+1 */
    int64_t *cursor;   /* n */
    uint32_t *tmp;     /* E */
    int64_t *ucnt;     /* n+1 */
    int64_t *row_ptr;  /* n+1 */
    int32_t *col;
} csr_ctx;

static int cmp_u32(const void *a, const void *b) {
    uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return (x > y) - (x < y);
}

static void sort_u32(uint32_t *a, int64_t k) {
    if (k <= 24) {
        for (int64_t i = 1; i < k; ++i) {
            uint32_t v = a[i];
            int64_t j = i - 1;
            while (j >= 0 && a[j] > v) { a[j + 1] = a[j]; --j; }
            a[j + 1] = v;
        }
    } else {
        qsort(a, (size_t)k, sizeof(uint32_t), cmp_u32);
    }
}

static void csr_count(void *c, int tid, int nt) {
    csr_ctx *x = (csr_ctx *)c;
    int64_t lo, hi;
    range_of(x->E, tid, nt, &lo, &hi);
    for (int64_t e = lo; e < hi; ++e)
        if (x->src[e] != x->dst[e]) __atomic_fetch_add(&x->cnt[x->src[e]], 1, __ATOMIC_RELAXED);
}

static void csr_scatter(void *c, int tid, int nt) {
    csr_ctx *x = (csr_ctx *)c;
    int64_t lo, hi;
    range_of(x->E, tid, nt, &lo, &hi);
    for (int64_t e = lo; e < hi; ++e) {
        uint32_t s = x->src[e];
        if (s == x->dst[e]) continue;
        int64_t pos = __atomic_fetch_add(&x->cursor[s], 1, __ATOMIC_RELAXED);
        x->tmp[pos] = x->dst[e];
    }
}

static void csr_sort_unique(void *c, int tid, int nt) {
    csr_ctx *x = (csr_ctx *)c;
    int64_t lo, hi;
    range_of(x->n, tid, nt, &lo, &hi);
    for (int64_t u = lo; u < hi; ++u) {
        uint32_t *r = x->tmp + x->cnt[u];
        int64_t k = x->cnt[u + 1] - x->cnt[u];
        sort_u32(r, k);
        int64_t q = 0;
        for (int64_t i = 0; i < k; ++i)
            if (q == 0 || r[i] != r[q - 1]) r[q++] = r[i];
        x->ucnt[u] = q;
    }
}

static void csr_compact(void *c, int tid, int nt) {
    csr_ctx *x = (csr_ctx *)c;
    int64_t lo, hi;
    range_of(x->n, tid, nt, &lo, &hi);
    for (int64_t u = lo; u < hi; ++u) {
        const uint32_t *r = x->tmp + x->cnt[u];
        int64_t base = x->row_ptr[u], k = x->row_ptr[u + 1] - base;
        for (int64_t i = 0; i < k; ++i) x->col[base + i] = (int32_t)r[i];
    }
}

/* Builds g->row_ptr / g->col from the (src, dst) list; self loops dropped,
 * duplicates removed, columns ascending.  Returns 0 on success. */
static int build_csr(gg_graph *g, int64_t n, int64_t E, const uint32_t *src,
                     const uint32_t *dst, int threads) {
    csr_ctx x;
    memset(&x, 0, sizeof(x));
    x.n = n; x.E = E; x.src = src; x.dst = dst;
    x.cnt = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
    x.cursor = (int64_t *)malloc(sizeof(int64_t) * ((size_t)n + 1));
    x.ucnt = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
    x.row_ptr = (int64_t *)malloc(sizeof(int64_t) * ((size_t)n + 1));
    if (!x.cnt || !x.cursor || !x.ucnt || !x.row_ptr) goto fail;
    parallel_for(threads, csr_count, &x);
    /* exclusive scan of counts, in place: cnt[u] becomes the row start */
    {
        int64_t run = 0;
        for (int64_t u = 0; u < n; ++u) { int64_t c = x.cnt[u]; x.cnt[u] = run; run += c; }
        x.cnt[n] = run;
        x.tmp = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)run + 1));
        if (!x.tmp) goto fail;
        memcpy(x.cursor, x.cnt, sizeof(int64_t) * (size_t)n);
    }
    parallel_for(threads, csr_scatter, &x);
    parallel_for(threads, csr_sort_unique, &x);
    {
        int64_t run = 0;
        x.row_ptr[0] = 0;
        for (int64_t u = 0; u < n; ++u) { run += x.ucnt[u]; x.row_ptr[u + 1] = run; }
        x.col = (int32_t *)malloc(sizeof(int32_t) * ((size_t)run + 1));
        if (!x.col) goto fail;
    }
    parallel_for(threads, csr_compact, &x);
    g->n = n;
    g->m = x.row_ptr[n];
    g->row_ptr = x.row_ptr;
    g->col = x.col;
    free(x.cnt); free(x.cursor); free(x.ucnt); free(x.tmp);
    return 0;
fail:
    free(x.cnt); free(x.cursor); free(x.ucnt); free(x.tmp); free(x.row_ptr); free(x.col);
    return -1;
}

static gg_graph *new_graph(void) {
    return (gg_graph *)calloc(1, sizeof(gg_graph));
}

/* ---------------- weights ---------------- */

typedef struct { gg_graph *g; uint64_t seed; double lo, hi; } w_ctx;

static void weights_fill(void *c, int tid, int nt) {
    w_ctx *x = (w_ctx *)c;
    int64_t lo, hi;
    range_of(x->g->n, tid, nt, &lo, &hi);
    for (int64_t u = lo; u < hi; ++u) {
        for (int64_t e = x->g->row_ptr[u]; e < x->g->row_ptr[u + 1]; ++e) {
            uint64_t key = ((uint64_t)u << 32) | (uint32_t)x->g->col[e];
            double U = (double)(rnd(x->seed, 7, key) >> 11) * (1.0 / 9007199254740992.0);
            x->g->w[e] = (float)(x->lo + (x->hi - x->lo) * U);
        }
    }
}

static int add_weights(gg_graph *g, uint64_t seed, double lo, double hi, int threads) {
    g->w = (float *)malloc(sizeof(float) * ((size_t)g->m + 1));
    if (!g->w) return -1;
    w_ctx x = {g, seed, lo, hi};
    parallel_for(threads, weights_fill, &x);
    return 0;
}

/* ---------------- Erdos-Renyi ---------------- */

gg_graph *gg_erdos_renyi(int64_t n, double p, double dangling_frac, uint64_t seed) {
    gg_graph *g = new_graph();
    if (!g) return NULL;
    const uint64_t t = thr64(p);
    /* forced-dangling nodes: first k of a seeded Fisher-Yates shuffle */
    int64_t k = (int64_t)llround((double)n * dangling_frac);
    if (k > n) k = n;
    unsigned char *dang = (unsigned char *)calloc((size_t)n + 1, 1);
    int64_t *perm = (int64_t *)malloc(sizeof(int64_t) * ((size_t)n + 1));
    g->row_ptr = (int64_t *)malloc(sizeof(int64_t) * ((size_t)n + 1));
    if (!dang || !perm || !g->row_ptr) goto fail;
    for (int64_t i = 0; i < n; ++i) perm[i] = i;
    for (int64_t i = 0; i < k; ++i) {
        int64_t j = i + (int64_t)(rnd(seed, 2, (uint64_t)i) % (uint64_t)(n - i));
        int64_t tmp = perm[i]; perm[i] = perm[j]; perm[j] = tmp;
        dang[perm[i]] = 1;
    }
    /* two passes: count, then fill */
    int64_t m = 0;
    g->row_ptr[0] = 0;
    for (int64_t u = 0; u < n; ++u) {
        if (!dang[u])
            for (int64_t v = 0; v < n; ++v)
                if (v != u && rnd(seed, 1, (uint64_t)(u * n + v)) < t) ++m;
        g->row_ptr[u + 1] = m;
    }
    g->col = (int32_t *)malloc(sizeof(int32_t) * ((size_t)m + 1));
    if (!g->col) goto fail;
    int64_t q = 0;
    for (int64_t u = 0; u < n; ++u)
        if (!dang[u])
            for (int64_t v = 0; v < n; ++v)
                if (v != u && rnd(seed, 1, (uint64_t)(u * n + v)) < t) g->col[q++] = (int32_t)v;
    g->n = n;
    g->m = m;
    free(dang); free(perm);
    return g;
fail:
    free(dang); free(perm);
    gg_free(g);
    return NULL;
}

/* ---------------- R-MAT ---------------- */

typedef struct {
    int scale;
    int64_t E;
    uint32_t ta, tab, tabc;
    uint64_t seed;
    uint32_t *src, *dst;
} rmat_ctx;

static void rmat_fill(void *c, int tid, int nt) {
    rmat_ctx *x = (rmat_ctx *)c;
    int64_t lo, hi;
    range_of(x->E, tid, nt, &lo, &hi);
    for (int64_t e = lo; e < hi; ++e) {
        uint32_t s = 0, d = 0;
        uint64_t r = 0;
        for (int l = 0; l < x->scale; ++l) {
            uint32_t u32;
            if ((l & 1) == 0) { r = rnd(x->seed, 3, ((uint64_t)e << 5) | (uint64_t)(l >> 1)); u32 = (uint32_t)r; }
            else u32 = (uint32_t)(r >> 32);
            uint32_t bs, bd;
            if (u32 < x->ta) { bs = 0; bd = 0; }
            else if (u32 < x->tab) { bs = 0; bd = 1; }
            else if (u32 < x->tabc) { bs = 1; bd = 0; }
            else { bs = 1; bd = 1; }
            s = (s << 1) | bs;
            d = (d << 1) | bd;
        }
        x->src[e] = s;
        x->dst[e] = d;
    }
}

gg_graph *gg_rmat(int scale, int edge_factor, double a, double b, double c,
                  int weighted, double wlo, double whi, uint64_t seed, int threads) {
    if (scale < 1 || scale > 31 || edge_factor < 0) return NULL;
    gg_graph *g = new_graph();
    if (!g) return NULL;
    const int64_t n = (int64_t)1 << scale;
    const int64_t E = (int64_t)edge_factor * n;
    rmat_ctx x;
    x.scale = scale; x.E = E; x.seed = seed;
    x.ta = thr32(a); x.tab = thr32(a + b); x.tabc = thr32(a + b + c);
    x.src = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)E + 1));
    x.dst = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)E + 1));
    if (!x.src || !x.dst) goto fail;
    parallel_for(threads, rmat_fill, &x);
    if (build_csr(g, n, E, x.src, x.dst, threads)) goto fail;
    free(x.src); free(x.dst);
    x.src = x.dst = NULL;
    if (weighted && add_weights(g, seed, wlo, whi, threads)) goto fail;
    return g;
fail:
    free(x.src); free(x.dst);
    gg_free(g);
    return NULL;
}

/* ---------------- stochastic block model ---------------- */

typedef struct {
    int64_t n;
    int blocks;
    const int64_t *bstart;   /* blocks+1 */
    const int32_t *bof;      /* n */
    const int64_t *perm;     /* n: old id -> new id */
    uint32_t t_in, t_out;
    uint64_t seed;
    const int64_t *eoff;     /* n+1: edge slots per node */
    uint32_t *src, *dst;
} sbm_ctx;

static int sbm_count(uint64_t seed, uint64_t s, int64_t u, uint32_t thr) {
    int k = 0;
    for (int j = 0; j < 32; ++j) {
        uint64_t r = rnd(seed, s, ((uint64_t)u << 5) | (uint64_t)j);
        k += ((uint32_t)r < thr) + ((uint32_t)(r >> 32) < thr);
    }
    return k;
}

static void sbm_fill(void *c, int tid, int nt) {
    sbm_ctx *x = (sbm_ctx *)c;
    int64_t lo, hi;
    range_of(x->n, tid, nt, &lo, &hi);
    for (int64_t u = lo; u < hi; ++u) {
        const int b = x->bof[u];
        const int64_t b0 = x->bstart[b], bs = x->bstart[b + 1] - b0;
        int64_t slot = x->eoff[u];
        const int k_in = sbm_count(x->seed, 4, u, x->t_in);
        const int k_out = sbm_count(x->seed, 5, u, x->t_out);
        for (int j = 0; j < k_in; ++j) {
            uint64_t r = rnd(x->seed, 6, ((uint64_t)u << 8) | (uint64_t)j);
            int64_t v = b0 + (int64_t)(r % (uint64_t)bs);
            x->src[slot] = (uint32_t)x->perm[u];
            x->dst[slot] = (uint32_t)x->perm[v];   /* v == u gives a self loop: dropped */
            ++slot;
        }
        const int64_t rest = x->n - bs;
        for (int j = 0; j < k_out; ++j) {
            int64_t v = u;
            if (rest > 0) {
                uint64_t r = rnd(x->seed, 8, ((uint64_t)u << 8) | (uint64_t)j);
                v = (int64_t)(r % (uint64_t)rest);
                if (v >= b0) v += bs;
            }
            x->src[slot] = (uint32_t)x->perm[u];
            x->dst[slot] = (uint32_t)x->perm[v];
            ++slot;
        }
    }
}

gg_graph *gg_sbm(int64_t n, int blocks, double zipf_s, double intra_mean,
                 double inter_mean, uint64_t seed, int threads) {
    if (n < 1 || blocks < 1 || blocks > n) return NULL;
    gg_graph *g = new_graph();
    if (!g) return NULL;
    int64_t *bstart = (int64_t *)malloc(sizeof(int64_t) * ((size_t)blocks + 1));
    int32_t *bof = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    int64_t *perm = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    int64_t *eoff = (int64_t *)malloc(sizeof(int64_t) * ((size_t)n + 1));
    uint32_t *src = NULL, *dst = NULL;
    if (!bstart || !bof || !perm || !eoff) goto fail;
    {
        /* Zipf sizes: floor(n * w_i / sum w), remainder to the largest blocks,
         * every block at least one node. */
        double tot = 0.0;
        for (int i = 0; i < blocks; ++i) tot += pow((double)(i + 1), -zipf_s);
        int64_t used = 0;
        int64_t *sz = (int64_t *)malloc(sizeof(int64_t) * (size_t)blocks);
        if (!sz) goto fail;
        for (int i = 0; i < blocks; ++i) {
            sz[i] = (int64_t)floor((double)n * pow((double)(i + 1), -zipf_s) / tot);
            if (sz[i] < 1) sz[i] = 1;
            used += sz[i];
        }
        int i = 0;
        while (used < n) { sz[i % blocks]++; used++; i++; }
        i = blocks - 1;
        while (used > n) { if (sz[i] > 1) { sz[i]--; used--; } i = (i == 0) ? blocks - 1 : i - 1; }
        bstart[0] = 0;
        for (int b = 0; b < blocks; ++b) bstart[b + 1] = bstart[b] + sz[b];
        free(sz);
    }
    for (int b = 0; b < blocks; ++b)
        for (int64_t v = bstart[b]; v < bstart[b + 1]; ++v) bof[v] = b;
    for (int64_t i = 0; i < n; ++i) perm[i] = i;
    for (int64_t i = n - 1; i > 0; --i) {
        int64_t j = (int64_t)(rnd(seed, 9, (uint64_t)i) % (uint64_t)(i + 1));
        int64_t t = perm[i]; perm[i] = perm[j]; perm[j] = t;
    }
    const uint32_t t_in = thr32(intra_mean / 64.0), t_out = thr32(inter_mean / 64.0);
    eoff[0] = 0;
    for (int64_t u = 0; u < n; ++u)
        eoff[u + 1] = eoff[u] + sbm_count(seed, 4, u, t_in) + sbm_count(seed, 5, u, t_out);
    const int64_t E = eoff[n];
    src = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)E + 1));
    dst = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)E + 1));
    if (!src || !dst) goto fail;
    sbm_ctx x = {n, blocks, bstart, bof, perm, t_in, t_out, seed, eoff, src, dst};
    parallel_for(threads, sbm_fill, &x);
    if (build_csr(g, n, E, src, dst, threads)) goto fail;
    g->block = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    if (!g->block) goto fail;
    for (int64_t v = 0; v < n; ++v) g->block[perm[v]] = bof[v];
    free(bstart); free(bof); free(perm); free(eoff); free(src); free(dst);
    return g;
fail:
    free(bstart); free(bof); free(perm); free(eoff); free(src); free(dst);
    gg_free(g);
    return NULL;
}

/* ---------------- accessors ---------------- */

int64_t gg_n(const gg_graph *g) { return g ? g->n : 0; }
int64_t gg_m(const gg_graph *g) { return g ? g->m : 0; }
int gg_weighted(const gg_graph *g) { return g && g->w; }

void gg_export(const gg_graph *g, int64_t *row_ptr, int32_t *col, float *w,
               int32_t *block_of) {
    if (!g) return;
    memcpy(row_ptr, g->row_ptr, sizeof(int64_t) * ((size_t)g->n + 1));
    if (g->m) memcpy(col, g->col, sizeof(int32_t) * (size_t)g->m);
    if (w && g->m) {
        if (g->w) memcpy(w, g->w, sizeof(float) * (size_t)g->m);
        else for (int64_t e = 0; e < g->m; ++e) w[e] = 1.0f;
    }
    if (block_of && g->block) memcpy(block_of, g->block, sizeof(int32_t) * (size_t)g->n);
}

void gg_free(gg_graph *g) {
    if (!g) return;
    free(g->row_ptr); free(g->col); free(g->w); free(g->block);
    free(g);
}

/* ---------------- seed sets ---------------- */

int64_t gg_seed_sets(int64_t n, const int64_t *row_ptr, int64_t nsets, int lo,
                     int hi, uint64_t seed, int64_t *seed_ptr, int32_t *seed_idx) {
    if (n < 1 || lo < 1 || hi < lo) return -1;
    const int64_t m = row_ptr[n];
    int64_t total = 0;
    seed_ptr[0] = 0;
    uint64_t ctr = 0;
    for (int64_t s = 0; s < nsets; ++s) {
        int64_t want = lo + (int64_t)(rnd(seed, 10, (uint64_t)s) % (uint64_t)(hi - lo + 1));
        if (want > n) want = n;
        int64_t got = 0;
        int64_t attempts = 0;
        while (got < want) {
            int64_t v;
            uint64_t r = rnd(seed, 11, ctr++);
            if (m > 0 && attempts < 64 * want) {
                /* a uniform edge's source: probability proportional to out-degree */
                int64_t e = (int64_t)(r % (uint64_t)m);
                int64_t a = 0, b = n;        /* largest u with row_ptr[u] <= e */
                while (b - a > 1) { int64_t mid = (a + b) / 2; if (row_ptr[mid] <= e) a = mid; else b = mid; }
                v = a;
            } else {
                v = (int64_t)(r % (uint64_t)n);
            }
            ++attempts;
            int dup = 0;
            for (int64_t k = 0; k < got; ++k)
                if (seed_idx[total + k] == (int32_t)v) { dup = 1; break; }
            if (!dup) seed_idx[total + got++] = (int32_t)v;
        }
        total += got;
        seed_ptr[s + 1] = total;
    }
    return total;
}
