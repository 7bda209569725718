// PageRank / personalized-PageRank power iteration on the in-edge CSR.
//
// The reference iterates x_{k+1} = F(x_k) in FP64 and stops at the first k
// with ||x_k - x_{k-1}||_1 < tol (src/pagerank.rs:142-180, src/ppr.rs:117-149).
// F is affine, F(x) = c + A x with
//     A x = d * (P^T x + (sum_{u dangling} x_u) * red),
// red = 1/n (uniform, src/pagerank.rs:150) or p (src/ppr.rs:125-128), and
// c = (1-d) * red.  So the step r_k = x_k - x_{k-1} obeys r_{k+1} = A r_k, and
// the library iterates on r (the "residual form"):
//   k = 1:  r_1 = F(x_0) - x_0              (x_0 = red)
//   k > 1:  r_k = A r_{k-1}
//   x_k = x_0 + r_1 + ... + r_k,  diff_k = ||r_k||_1 (the reference's diff_l1)
// Each step is one pull kernel over the in-edge CSR (K3): every row v gathers
// the previous step's vector at its in-neighbours, and the same kernel fuses
// the dangling sum, the L1 norm (K4) and the accumulation of x.
//
// Precision.  While ||r||_1 >= theta (first few steps) the gathered vector and
// all arithmetic are double-float (two FP32 words, ~48 bits); afterwards the
// gathered vector is FP32 and the steps are summed into an FP32 tail.  x is
// then acc (double-float) + tail, formed in FP64 at the end.  The global sums
// (dangling mass, L1 norm) are exact 64-bit fixed-point integer sums, so they
// are independent of summation order and bit-reproducible.
//
// Data movement.  One block per SM walks its batches (see objects.cuh) in a
// ring of kStages shared-memory stages: one thread issues bulk asynchronous
// copies (TMA) of a batch's column indices, weights and row offsets several
// batches ahead, completing on an mbarrier, so the edge streams never wait on
// the threads.  The threads gather the previous step's vector at the staged
// column indices; its first kHot entries -- the most gathered nodes after the
// in-degree relabelling -- are staged in shared memory at kernel start.
// Segment batches give each row sw lanes (an xor-shuffle reduction); chunks of
// big rows are reduced by the whole block and combined, in chunk order, by the
// chunk that finishes last.
//
// Convergence is decided on the device: the kernel for step k first reads
// diff_{k-1}; if it is below tol (or k-1 == max_iterations) it records the
// run and every block returns, so the host may launch steps ahead.
#include <algorithm>
#include <cmath>
#include <vector>

#include "objects.cuh"

namespace gops {

enum Mode : int { kPlain = 0, kWeighted = 1, kPpr = 2 };

constexpr int kThreads = 256;  // init / small kernels
constexpr int kWarps = kThreads / kWarp;
constexpr int kPullWarps = kPullThreads / kWarp;
constexpr int kStages = 3;
#ifndef GOPS_HOT
#define GOPS_HOT 26624
#endif
constexpr int kHot = GOPS_HOT;   // FP32 entries of the gathered vector staged per block
constexpr double kTheta = 1e-2;  // double-float phase while ||r||_1 >= kTheta

// shared-memory stage of one batch
struct Stage {
  int32_t col[kBatchEdges + 8];
  float val[kBatchEdges + 8];
  long long rp[kPullThreads + 4];
};

struct BatchDesc {
  int kind;         // 0: segment rows, 1: chunk of a big row
  int row0, nrows;  // segment rows / the big row (row0)
  int sw;           // lanes per row (segment batches)
  int e0a;          // first staged edge (16-byte aligned)
  int rpa;          // first staged row offset (16-byte aligned)
  int cs, ce;       // chunk edge range (big rows)
  int first, nch;   // chunk batches of the big row
};

struct IterParams {
  int64_t n;
  const int64_t *rp;
  const int32_t *col;
  const float *val;
  const float *deg;
  const uint32_t *dmask;
  const int32_t *big_first;
  const int32_t *big_batch_row;
  Plan plan;
  const float2 *gdf_in;
  float2 *gdf_out;
  const float *gf_in;
  float *gf_out;
  float2 *acc;
  float *tail;
  const float2 *pdf;
  long long *sums;
  SolveState *st;
  float2 *lpart;
  unsigned *lcnt;
  int *err;
  df d, omd, inv_n;
  float fx_scale;
  double fx_inv;
  double tol, theta;
  unsigned long long k, max_iter;
};

// --------------------------------------------------------------------------
// precision policies
// --------------------------------------------------------------------------
struct PrecDF {
  using T = df;
  static constexpr bool kDF = true;
  static constexpr int kCached = kHot / 2;  // double-float entries staged in shared memory
  __device__ static T zero() { return {0.0f, 0.0f}; }
  __device__ static T add(T a, T b) { return df_add(a, b); }
  __device__ static T shfl(T v, int m) { return shfl_xor_df(v, m, 32); }
  __device__ static T load_g(const IterParams &p, const void *cache, int32_t u) {
    float2 g;
    if (u < kCached) g = reinterpret_cast<const float2 *>(cache)[u];
    else g = __ldg(&p.gdf_in[u]);
    return {g.x, g.y};
  }
  __device__ static void stage(const IterParams &p, void *cache) {
    float2 *c = reinterpret_cast<float2 *>(cache);
    const int lim = (int)(p.n < (int64_t)kCached ? p.n : (int64_t)kCached);
    for (int i = threadIdx.x; i < lim; i += blockDim.x) c[i] = __ldg(&p.gdf_in[i]);
  }
  __device__ static T scale(T g, float w) { return df_mul_f(g, w); }
  __device__ static float2 pack(T v) { return make_float2(v.hi, v.lo); }
  __device__ static T unpack(float2 v) { return {v.x, v.y}; }
};

struct PrecF32 {
  using T = float;
  static constexpr bool kDF = false;
  static constexpr int kCached = kHot;
  __device__ static T zero() { return 0.0f; }
  __device__ static T add(T a, T b) { return a + b; }
  __device__ static T shfl(T v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
  __device__ static T load_g(const IterParams &p, const void *cache, int32_t u) {
    if (u < kCached) return reinterpret_cast<const float *>(cache)[u];
    return __ldg(&p.gf_in[u]);
  }
  __device__ static void stage(const IterParams &p, void *cache) {
    float *c = reinterpret_cast<float *>(cache);
    const int lim = (int)(p.n < (int64_t)kCached ? p.n : (int64_t)kCached);
    for (int i = threadIdx.x; i < lim; i += blockDim.x) c[i] = __ldg(&p.gf_in[i]);
  }
  __device__ static T scale(T g, float w) { return g * w; }
  __device__ static float2 pack(T v) { return make_float2(v, 0.0f); }
  __device__ static T unpack(float2 v) { return v.x; }
};

struct Acc {
  long long l1 = 0, dang = 0;
  int bad = 0;
};

// Per-row inputs of the epilogue, loaded before the row's edges so their
// latency overlaps the gathers: the running x part (acc in the double-float
// phase, tail in the FP32 phase), the out-degree, the dangling flag and the
// personalization entry.
struct RowIn {
  float2 x;
  float2 red;
  float deg;
  int dang;
};

template <class P, int MODE>
__device__ __forceinline__ RowIn row_in(const IterParams &p, int64_t v) {
  RowIn in;
  if constexpr (P::kDF) in.x = p.acc[v];
  else in.x = make_float2(p.tail[v], 0.0f);
  in.red = (MODE == kPpr) ? p.pdf[v] : make_float2(p.inv_n.hi, p.inv_n.lo);
  if (MODE == kWeighted) {
    in.deg = 1.0f;
    in.dang = (__ldg(&p.dmask[v >> 5]) >> (v & 31)) & 1u;
  } else {
    in.deg = __ldg(&p.deg[v]);
    in.dang = in.deg == 0.0f;
  }
  return in;
}

// Row v's new step value from its gathered sum s.
template <int MODE>
__device__ __forceinline__ void epilogue_df(const IterParams &p, int64_t v, df s, df dsum,
                                            const RowIn &in, Acc &a) {
  const df red = {in.red.x, in.red.y};
  df r = df_mul(p.d, df_add(s, df_mul(dsum, red)));
  if (p.k == 1) r = df_add(df_add(df_mul(p.omd, red), r), df_neg(red));  // F(x_0) - x_0
  const df an = df_add({in.x.x, in.x.y}, r);
  p.acc[v] = make_float2(an.hi, an.lo);
  const df ar = r.hi < 0.0f ? df_neg(r) : r;
  a.l1 += fx_of(ar.hi, p.fx_scale) + fx_of(ar.lo, p.fx_scale);
  a.bad |= !isfinite(r.hi);
  if (in.dang) a.dang += fx_of(r.hi, p.fx_scale) + fx_of(r.lo, p.fx_scale);
  df g = r;
  if (MODE != kWeighted) g = in.deg > 0.0f ? df_div_f(r, in.deg) : df{0.0f, 0.0f};
  p.gdf_out[v] = make_float2(g.hi, g.lo);
  p.gf_out[v] = g.hi;
}

template <int MODE>
__device__ __forceinline__ void epilogue_f32(const IterParams &p, int64_t v, float s, float dsum,
                                             const RowIn &in, Acc &a) {
  const float r = p.d.hi * (s + dsum * in.red.x);
  p.tail[v] = in.x.x + r;
  a.l1 += fx_of(fabsf(r), p.fx_scale);
  a.bad |= !isfinite(r);
  if (in.dang) a.dang += fx_of(r, p.fx_scale);
  float g = r;
  if (MODE != kWeighted) g = in.deg > 0.0f ? __fdiv_rn(r, in.deg) : 0.0f;
  p.gf_out[v] = g;
}

template <class P, int MODE>
__device__ __forceinline__ void epilogue(const IterParams &p, int64_t v, typename P::T s, df dsum,
                                         const RowIn &in, Acc &a) {
  if constexpr (P::kDF) epilogue_df<MODE>(p, v, s, dsum, in, a);
  else epilogue_f32<MODE>(p, v, s, dsum.hi, in, a);
}

// Reads diff_{k-1}; decides whether the run is over and whether this kernel's
// precision is the active one.  Returns false when the block should exit.
template <bool WANT_DF>
__device__ bool prologue(const IterParams &p, df *dsum) {
  const unsigned long long k = p.k;
  if (*(volatile int *)&p.st->done) return false;  // recorded by an earlier step
  const int prev = (int)((k - 1) % 3);
  double diff = INFINITY;
  if (k > 1) {
    const long long raw = *(volatile long long *)&p.sums[prev * 4 + 1];
    const long long badc = *(volatile long long *)&p.sums[prev * 4 + 2];
    diff = badc ? NAN : (double)raw * p.fx_inv;
  }
  const bool conv = k > 1 && diff < p.tol;
  if (conv || k - 1 >= p.max_iter) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      p.st->done = 1;
      p.st->converged = conv ? 1 : 0;
      p.st->iterations = k - 1;
      p.st->diff_l1 = diff;
    }
    return false;
  }
  const bool f32 = k > 1 && (*(volatile int *)&p.st->f32_phase || diff < p.theta);
  if (f32 == WANT_DF) return false;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    p.st->f32_phase = f32 ? 1 : 0;
    if (f32 && p.st->f32_from == 0) p.st->f32_from = k;
    const int nxt = (int)((k + 1) % 3);
    for (int i = 0; i < 4; ++i) p.sums[nxt * 4 + i] = 0;
  }
  const long long draw = *(volatile long long *)&p.sums[prev * 4 + 0];
  *dsum = df_from_double((double)draw * p.fx_inv);
  return true;
}

// Producer side: describes batch b and starts its bulk copies into stage st,
// completing on bar.  Called by one thread.  Copies start and end on 16-byte
// boundaries (the edge and row-offset arrays carry padding past their ends).
template <int MODE>
__device__ void issue_batch(const IterParams &p, int b, Stage &st, BatchDesc &dsc, uint64_t *bar) {
  uint32_t rp_bytes = 0;
  int e0a, e1a;
  if (b < p.plan.n_big_batches) {
    const int h = __ldg(&p.big_batch_row[b]);
    const int first = __ldg(&p.big_first[h]);
    const int rb = (int)__ldg(&p.rp[h]), re = (int)__ldg(&p.rp[h + 1]);
    const int cs = rb + (b - first) * kBatchEdges;
    const int ce = min(re, cs + kBatchEdges);
    e0a = cs & ~3;
    e1a = (ce + 3) & ~3;
    dsc.kind = 1;
    dsc.row0 = h;
    dsc.nrows = 1;
    dsc.sw = 32;
    dsc.rpa = 0;
    dsc.cs = cs;
    dsc.ce = ce;
    dsc.first = first;
    dsc.nch = __ldg(&p.big_first[h + 1]) - first;
  } else {
    int si = 0;
    while (si + 1 < p.plan.n_segs && b >= p.plan.segs[si + 1].batch_begin) ++si;
    const Segment &sg = p.plan.segs[si];
    const int r0 = sg.row_begin + (b - sg.batch_begin) * sg.rows_per_batch;
    const int nr = min(sg.rows_per_batch, sg.row_end - r0);
    const int e0 = (int)__ldg(&p.rp[r0]), e1 = (int)__ldg(&p.rp[r0 + nr]);
    e0a = e0 & ~3;
    e1a = (e1 + 3) & ~3;
    const int rpa = r0 & ~1, rpe = (r0 + nr + 2) & ~1;  // covers rp[r0 .. r0+nr]
    dsc.kind = 0;
    dsc.row0 = r0;
    dsc.nrows = nr;
    dsc.sw = sg.sw;
    dsc.rpa = rpa;
    rp_bytes = (uint32_t)(rpe - rpa) * 8u;
  }
  dsc.e0a = e0a;
  const uint32_t eb = (uint32_t)(e1a - e0a) * 4u;
  mbar_arrive_expect_tx(bar, rp_bytes + eb * (MODE == kWeighted ? 2u : 1u));
  if (rp_bytes) bulk_g2s(st.rp, p.rp + dsc.rpa, rp_bytes, bar);
  if (eb) {
    bulk_g2s(st.col, p.col + e0a, eb, bar);
    if (MODE == kWeighted) bulk_g2s(st.val, p.val + e0a, eb, bar);
  }
}

// The pull kernel of step k in precision P (see the file comment).
template <class P, int MODE>
__global__ void __launch_bounds__(kPullThreads, 1) pull_kernel(IterParams p) {
  using T = typename P::T;
  extern __shared__ __align__(128) unsigned char smem[];
  Stage *stages = reinterpret_cast<Stage *>(smem);
  void *cache = smem + sizeof(Stage) * kStages;
  __shared__ uint64_t full[kStages];
  __shared__ BatchDesc desc[kStages];
  __shared__ T wred[kPullWarps];
  __shared__ long long bred[2][kPullWarps];
  __shared__ int bbad[kPullWarps];

  df dsum;
  if (!prologue<P::kDF>(p, &dsum)) return;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int nb = p.plan.n_batches;
  // the batches of this block are blockIdx.x + j * gridDim.x, j = 0, 1, ...
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&full[s], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0)
    for (int j = 0; j < kStages; ++j) {
      const int b = blockIdx.x + j * gridDim.x;
      if (b < nb) issue_batch<MODE>(p, b, stages[j], desc[j], &full[j]);
    }
  P::stage(p, cache);  // hot prefix of the gathered vector, while the copies fly
  __syncthreads();

  Acc a;
  for (int j = 0;; ++j) {
    const int b = blockIdx.x + j * gridDim.x;
    if (b >= nb) break;
    const int s = j % kStages;
    const bool ok = mbar_wait(&full[s], (uint32_t)((j / kStages) & 1));
    if (!__syncthreads_and(ok)) {
      // a bounded wait ran out: record it, let the copies already issued
      // land (bounded again), and leave
      if (tid == 0) {
        atomicOr(p.err, 1);
        for (int jj = j; jj < j + kStages; ++jj)
          if ((int)blockIdx.x + jj * (int)gridDim.x < nb)
            mbar_wait(&full[jj % kStages], (uint32_t)((jj / kStages) & 1));
      }
      break;
    }
    const Stage &stg = stages[s];
    const BatchDesc dsc = desc[s];
    if (dsc.kind == 0) {
      const int sw = dsc.sw;
      const int lg = 31 - __clz(sw);
      const int rr = tid >> lg, li = tid & (sw - 1);
      const bool valid = rr < dsc.nrows;
      const int64_t row = (int64_t)dsc.row0 + rr;
      RowIn in;
      if (valid && li == 0) in = row_in<P, MODE>(p, row);
      int eb = 0, ee = 0;
      if (valid) {
        eb = (int)(stg.rp[dsc.row0 - dsc.rpa + rr] - dsc.e0a);
        ee = (int)(stg.rp[dsc.row0 - dsc.rpa + rr + 1] - dsc.e0a);
      }
      T sum = P::zero();
      for (int e = eb + li; e < ee; e += 4 * sw) {
        const bool o1 = e + sw < ee, o2 = e + 2 * sw < ee, o3 = e + 3 * sw < ee;
        const int32_t c0 = stg.col[e];
        const int32_t c1 = o1 ? stg.col[e + sw] : 0;
        const int32_t c2 = o2 ? stg.col[e + 2 * sw] : 0;
        const int32_t c3 = o3 ? stg.col[e + 3 * sw] : 0;
        const T g0 = P::load_g(p, cache, c0);
        const T g1 = o1 ? P::load_g(p, cache, c1) : P::zero();
        const T g2 = o2 ? P::load_g(p, cache, c2) : P::zero();
        const T g3 = o3 ? P::load_g(p, cache, c3) : P::zero();
        if (MODE == kWeighted) {
          sum = P::add(sum, P::scale(g0, stg.val[e]));
          if (o1) sum = P::add(sum, P::scale(g1, stg.val[e + sw]));
          if (o2) sum = P::add(sum, P::scale(g2, stg.val[e + 2 * sw]));
          if (o3) sum = P::add(sum, P::scale(g3, stg.val[e + 3 * sw]));
        } else {
          sum = P::add(sum, g0);
          if (o1) sum = P::add(sum, g1);
          if (o2) sum = P::add(sum, g2);
          if (o3) sum = P::add(sum, g3);
        }
      }
      for (int o = sw >> 1; o > 0; o >>= 1) sum = P::add(sum, P::shfl(sum, o));
      if (valid && li == 0) epilogue<P, MODE>(p, row, sum, dsum, in, a);
    } else {
      // chunk [cs, ce) of big row row0, reduced by the whole block
      const int lo = dsc.cs - dsc.e0a, hi = dsc.ce - dsc.e0a;
      T sum = P::zero();
      for (int e = lo + tid; e < hi; e += 4 * kPullThreads) {
        const int e1 = e + kPullThreads, e2 = e + 2 * kPullThreads, e3 = e + 3 * kPullThreads;
        const bool o1 = e1 < hi, o2 = e2 < hi, o3 = e3 < hi;
        const T g0 = P::load_g(p, cache, stg.col[e]);
        const T g1 = o1 ? P::load_g(p, cache, stg.col[e1]) : P::zero();
        const T g2 = o2 ? P::load_g(p, cache, stg.col[e2]) : P::zero();
        const T g3 = o3 ? P::load_g(p, cache, stg.col[e3]) : P::zero();
        if (MODE == kWeighted) {
          sum = P::add(sum, P::scale(g0, stg.val[e]));
          if (o1) sum = P::add(sum, P::scale(g1, stg.val[e1]));
          if (o2) sum = P::add(sum, P::scale(g2, stg.val[e2]));
          if (o3) sum = P::add(sum, P::scale(g3, stg.val[e3]));
        } else {
          sum = P::add(sum, g0);
          if (o1) sum = P::add(sum, g1);
          if (o2) sum = P::add(sum, g2);
          if (o3) sum = P::add(sum, g3);
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) sum = P::add(sum, P::shfl(sum, o));
      if (lane == 0) wred[wid] = sum;
      __syncthreads();
      if (tid == 0) {
        T tot = wred[0];
        for (int w = 1; w < kPullWarps; ++w) tot = P::add(tot, wred[w]);
        const int h = dsc.row0;
        if (dsc.nch == 1) {
          const RowIn in = row_in<P, MODE>(p, h);
          epilogue<P, MODE>(p, h, tot, dsum, in, a);
        } else {
          p.lpart[b] = P::pack(tot);
          __threadfence();
          const unsigned tk = atomicAdd(&p.lcnt[h], 1u);
          if (tk == (unsigned)(dsc.nch - 1)) {
            __threadfence();
            T all = P::zero();
            for (int q = 0; q < dsc.nch; ++q) all = P::add(all, P::unpack(__ldcg(&p.lpart[dsc.first + q])));
            p.lcnt[h] = 0;
            const RowIn in = row_in<P, MODE>(p, h);
            epilogue<P, MODE>(p, h, all, dsum, in, a);
          }
        }
      }
    }
    __syncthreads();  // stage s is free again
    if (tid == 0) {
      const int bn = blockIdx.x + (j + kStages) * gridDim.x;
      if (bn < nb) {
        fence_proxy_async_smem();
        issue_batch<MODE>(p, bn, stages[s], desc[s], &full[s]);
      }
    }
  }

  // ---- block totals of the exact fixed-point sums -> one atomic each
  long long l1 = warp_sum_ll(a.l1), dg = warp_sum_ll(a.dang);
  int bad = warp_or(a.bad);
  if (lane == 0) { bred[0][wid] = l1; bred[1][wid] = dg; bbad[wid] = bad; }
  __syncthreads();
  if (tid == 0) {
    long long t1 = 0, t2 = 0;
    int tb = 0;
    for (int w = 0; w < kPullWarps; ++w) { t1 += bred[0][w]; t2 += bred[1][w]; tb |= bbad[w]; }
    const int cur = (int)(p.k % 3);
    atomicAdd((unsigned long long *)&p.sums[cur * 4 + 1], (unsigned long long)t1);
    atomicAdd((unsigned long long *)&p.sums[cur * 4 + 0], (unsigned long long)t2);
    if (tb) atomicAdd((unsigned long long *)&p.sums[cur * 4 + 2], 1ull);
  }
}

// x_0 = red, acc = x_0, tail = 0, gathered vector for step 1, sum_dangling x_0.
template <int MODE>
__global__ void __launch_bounds__(kThreads) init_kernel(IterParams p) {
  __shared__ long long bred[kWarps];
  long long dang = 0;
  for (int64_t v = (int64_t)blockIdx.x * kThreads + threadIdx.x; v < p.n;
       v += (int64_t)gridDim.x * kThreads) {
    const df red = (MODE == kPpr) ? PrecDF::unpack(p.pdf[v]) : p.inv_n;
    p.acc[v] = make_float2(red.hi, red.lo);
    p.tail[v] = 0.0f;
    df g = red;
    bool dang_v;
    if (MODE != kWeighted) {
      const float dg = p.deg[v];
      dang_v = dg == 0.0f;
      g = dang_v ? df{0.0f, 0.0f} : df_div_f(red, dg);
    } else {
      dang_v = (p.dmask[v >> 5] >> (v & 31)) & 1u;
    }
    if (dang_v) dang += fx_of(red.hi, p.fx_scale) + fx_of(red.lo, p.fx_scale);
    p.gdf_out[v] = make_float2(g.hi, g.lo);
    p.gf_out[v] = g.hi;
  }
  dang = warp_sum_ll(dang);
  if ((threadIdx.x & 31) == 0) bred[threadIdx.x >> 5] = dang;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long t = 0;
    for (int w = 0; w < kWarps; ++w) t += bred[w];
    atomicAdd((unsigned long long *)&p.sums[0], (unsigned long long)t);
  }
}

// x in original node order: x[perm[i]] = acc[i] + tail[i].
__global__ void finalize_kernel(int64_t n, const float2 *acc, const float *tail, const int32_t *perm,
                                double *x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[perm[i]] = (double)acc[i].x + (double)acc[i].y + (double)tail[i];
}

// Personalization into relabelled order: dst[i] = src[perm[i]].
__global__ void permute_pdf(int64_t n, const float2 *src, const int32_t *perm, float2 *dst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[perm[i]];
}

// --------------------------------------------------------------------------
// host side
// --------------------------------------------------------------------------
void workspace_free(Workspace &ws) {
  cudaFree(ws.gdf[0]); cudaFree(ws.gdf[1]); cudaFree(ws.gf[0]); cudaFree(ws.gf[1]);
  cudaFree(ws.acc); cudaFree(ws.tail); cudaFree(ws.pdf); cudaFree(ws.scores);
  cudaFree(ws.sums); cudaFree(ws.lpart); cudaFree(ws.lcnt); cudaFree(ws.state); cudaFree(ws.err);
  ws = Workspace{};
}

Status workspace_ensure(Ctx *ctx, Graph *g) {
  (void)ctx;
  Workspace &ws = g->ws;
  if (ws.sums) return Status::ok();
  const size_t n = (size_t)std::max<int64_t>(g->n, 1);
  const size_t nbb = (size_t)std::max<int32_t>(g->plan.n_big_batches, 1);
  const size_t nbig = (size_t)std::max<int32_t>(g->plan.n_big, 1);
  GOPS_CUDA_TRY(cudaMalloc(&ws.gdf[0], sizeof(float2) * n));
  GOPS_CUDA_TRY(cudaMalloc(&ws.gdf[1], sizeof(float2) * n));
  GOPS_CUDA_TRY(cudaMalloc(&ws.gf[0], sizeof(float) * n));
  GOPS_CUDA_TRY(cudaMalloc(&ws.gf[1], sizeof(float) * n));
  GOPS_CUDA_TRY(cudaMalloc(&ws.acc, sizeof(float2) * n));
  GOPS_CUDA_TRY(cudaMalloc(&ws.tail, sizeof(float) * n));
  GOPS_CUDA_TRY(cudaMalloc(&ws.pdf, sizeof(float2) * n));
  GOPS_CUDA_TRY(cudaMalloc(&ws.scores, sizeof(double) * n));
  GOPS_CUDA_TRY(cudaMalloc(&ws.lpart, sizeof(float2) * nbb));
  GOPS_CUDA_TRY(cudaMalloc(&ws.lcnt, sizeof(unsigned) * nbig));
  GOPS_CUDA_TRY(cudaMalloc(&ws.state, sizeof(SolveState)));
  GOPS_CUDA_TRY(cudaMalloc(&ws.sums, sizeof(long long) * 12));
  GOPS_CUDA_TRY(cudaMalloc(&ws.err, sizeof(int)));
  ws.n = g->n;
  return Status::ok();
}

namespace {

constexpr size_t kPullSmem = sizeof(Stage) * kStages + sizeof(float) * kHot;

template <class P, int MODE>
Status pull_grid(const Ctx *ctx, const Graph *g, int *grid) {
  GOPS_CUDA_TRY(cudaFuncSetAttribute(pull_kernel<P, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kPullSmem));
  int occ = 0;
  GOPS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pull_kernel<P, MODE>, kPullThreads,
                                                              kPullSmem));
  occ = std::max(1, occ);
  *grid = (int)std::max<int64_t>(
      1, std::min<int64_t>(std::max<int32_t>(g->plan.n_batches, 1), (int64_t)ctx->num_sms * occ));
  return Status::ok();
}

template <int MODE>
Status run_mode(Ctx *ctx, Graph *g, const gops_config *cfg, double pv_l1, gops_run *run) {
  cudaStream_t s = ctx->stream;
  Workspace &ws = g->ws;
  IterParams p{};
  p.n = g->n;
  p.rp = g->in_rp;
  p.col = g->in_col;
  p.val = g->in_val;
  p.deg = g->deg;
  p.dmask = g->dmask_w;
  p.big_first = g->big_first;
  p.big_batch_row = g->big_batch_row;
  p.plan = g->plan;
  p.acc = ws.acc;
  p.tail = ws.tail;
  p.pdf = ws.pdf;
  p.sums = ws.sums;
  p.st = ws.state;
  p.lpart = ws.lpart;
  p.lcnt = ws.lcnt;
  p.err = ws.err;
  p.d = df_from_double(cfg->damping);
  p.omd = df_from_double(1.0 - cfg->damping);
  p.inv_n = df_from_double(1.0 / (double)g->n);
  int e = 0;
  while (e < 20 && std::ldexp(1.0, e) < std::max(1.0, pv_l1)) ++e;
  const int F = 58 - 2 * e;
  p.fx_scale = std::ldexp(1.0f, F);
  p.fx_inv = std::ldexp(1.0, -F);
  p.tol = cfg->tolerance;
  p.theta = kTheta;
  p.max_iter = cfg->max_iterations;

  GOPS_CUDA_TRY(cudaMemsetAsync(ws.sums, 0, sizeof(long long) * 12, s));
  GOPS_CUDA_TRY(cudaMemsetAsync(ws.state, 0, sizeof(SolveState), s));
  GOPS_CUDA_TRY(cudaMemsetAsync(ws.err, 0, sizeof(int), s));
  GOPS_CUDA_TRY(cudaMemsetAsync(ws.lcnt, 0, sizeof(unsigned) * std::max<int32_t>(g->plan.n_big, 1), s));
  GOPS_CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  uint64_t launches = 0;
  // step 0
  p.k = 0;
  p.gdf_out = ws.gdf[0];
  p.gf_out = ws.gf[0];
  const int init_grid = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div<int64_t>(g->n, kThreads),
                                                                     (int64_t)ctx->num_sms * 8));
  init_kernel<MODE><<<init_grid, kThreads, 0, s>>>(p);
  GOPS_CUDA_TRY(cudaGetLastError());
  ++launches;
  GOPS_CUDA_TRY(cudaEventRecord(ctx->ev[1], s));

  int grid_df = 1, grid_f = 1;
  GOPS_TRY((pull_grid<PrecDF, MODE>(ctx, g, &grid_df)));
  GOPS_TRY((pull_grid<PrecF32, MODE>(ctx, g, &grid_f)));
  bool f32_known = false;
  unsigned long long k = 1;
  const int chunk = 4;
  // per-launch timing: (step, is_df) of every timed launch, events 2i / 2i+1
  std::vector<std::pair<unsigned long long, bool>> timed;
  auto timed_launch = [&](bool is_df) -> Status {
    if (!ctx->timing) return Status::ok();
    const size_t need = 2 * (timed.size() + 1);
    while (ctx->tev.size() < need) {
      cudaEvent_t ev;
      GOPS_CUDA_TRY(cudaEventCreate(&ev));
      ctx->tev.push_back(ev);
    }
    timed.push_back({k, is_df});
    return Status::ok();
  };
  for (;;) {
    for (int j = 0; j < chunk && k - 1 <= cfg->max_iterations; ++j, ++k) {
      p.k = k;
      p.gdf_in = ws.gdf[(k - 1) & 1];
      p.gf_in = ws.gf[(k - 1) & 1];
      p.gdf_out = ws.gdf[k & 1];
      p.gf_out = ws.gf[k & 1];
      if (!f32_known) {
        GOPS_TRY(timed_launch(true));
        if (ctx->timing) GOPS_CUDA_TRY(cudaEventRecord(ctx->tev[2 * timed.size() - 2], s));
        pull_kernel<PrecDF, MODE><<<grid_df, kPullThreads, kPullSmem, s>>>(p);
        if (ctx->timing) GOPS_CUDA_TRY(cudaEventRecord(ctx->tev[2 * timed.size() - 1], s));
        ++launches;
      }
      if (k >= 2) {
        GOPS_TRY(timed_launch(false));
        if (ctx->timing) GOPS_CUDA_TRY(cudaEventRecord(ctx->tev[2 * timed.size() - 2], s));
        pull_kernel<PrecF32, MODE><<<grid_f, kPullThreads, kPullSmem, s>>>(p);
        if (ctx->timing) GOPS_CUDA_TRY(cudaEventRecord(ctx->tev[2 * timed.size() - 1], s));
        ++launches;
      }
    }
    GOPS_CUDA_TRY(cudaGetLastError());
    GOPS_CUDA_TRY(cudaMemcpyAsync(ctx->host_state, ws.state, sizeof(SolveState),
                                  cudaMemcpyDeviceToHost, s));
    GOPS_CUDA_TRY(cudaStreamSynchronize(s));
    if (ctx->host_state->done) break;
    if (ctx->host_state->f32_phase) f32_known = true;
    if (k - 1 > cfg->max_iterations)
      return Status{GOPS_ERR_INTERNAL, "solver did not record completion"};
  }
  int err = 0;
  GOPS_CUDA_TRY(cudaMemcpyAsync(&err, ws.err, sizeof(int), cudaMemcpyDeviceToHost, s));
  GOPS_CUDA_TRY(cudaEventRecord(ctx->ev[2], s));
  finalize_kernel<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div<int64_t>(g->n, 256), 4096)),
                    256, 0, s>>>(g->n, ws.acc, ws.tail, g->perm, ws.scores);
  GOPS_CUDA_TRY(cudaGetLastError());
  ++launches;
  GOPS_CUDA_TRY(cudaEventRecord(ctx->ev[3], s));
  GOPS_CUDA_TRY(cudaEventSynchronize(ctx->ev[3]));
  if (err) return Status{GOPS_ERR_TIMEOUT, "a bounded device wait ran out in the pull kernel"};
  run->iterations = ctx->host_state->iterations;
  run->diff_l1 = ctx->host_state->diff_l1;
  run->converged = ctx->host_state->converged;
  run->reserved = 0;
  float t_all = 0.f, t_it = 0.f;
  cudaEventElapsedTime(&t_all, ctx->ev[0], ctx->ev[3]);
  cudaEventElapsedTime(&t_it, ctx->ev[1], ctx->ev[2]);
  ctx->stats.solve_ms = t_all;
  ctx->stats.iterate_ms = t_it;
  if (ctx->timing) {
    // launches that did the work of a step (not the ones that found the run
    // finished or the other precision active)
    const unsigned long long its = ctx->host_state->iterations;
    const unsigned long long f32_from = ctx->host_state->f32_from;
    for (size_t i = 0; i < timed.size(); ++i) {
      const unsigned long long kk = timed[i].first;
      const bool is_df = timed[i].second;
      const bool active =
          kk <= its && (is_df ? (f32_from == 0 || kk < f32_from) : (f32_from && kk >= f32_from));
      if (!active) continue;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ctx->tev[2 * i], ctx->tev[2 * i + 1]);
      if (is_df) { ctx->stats.df_ms += ms; ctx->stats.df_launches++; }
      else { ctx->stats.f32_ms += ms; ctx->stats.f32_launches++; }
    }
  }
  ctx->stats.kernel_launches += launches;
  ctx->stats.iterations = run->iterations;
  return Status::ok();
}

}  // namespace

// mode: 0 plain, 1 weighted, 2 personalized (p_host: n raw entries)
Status solve(Ctx *ctx, Graph *g, const gops_config *cfg, int mode, const double *p_host,
             double *scores_host, gops_run *run) {
  ctx->stats = gops_stats{};
  if (g->n == 0) {  // src/pagerank.rs:123-131, src/ppr.rs:96-103
    run->iterations = 0;
    run->diff_l1 = 0.0;
    run->converged = 1;
    run->reserved = 0;
    return Status::ok();
  }
  if (mode == kWeighted && !g->weighted)
    return Status{GOPS_ERR_INVALID, "graph was uploaded without weights"};
  GOPS_TRY(workspace_ensure(ctx, g));
  double pv_l1 = 1.0;
  if (mode == kPpr) {
    // normalisation of src/ppr.rs:104-109, sequential FP64 like the reference
    const int64_t n = g->n;
    double psum = 0.0;
    for (int64_t i = 0; i < n; ++i) psum += p_host[i];
    std::vector<float2> pdf((size_t)n);
    pv_l1 = 0.0;
    for (int64_t i = 0; i < n; ++i) {
      const double v = psum > 0.0 ? p_host[i] / psum : 1.0 / (double)n;
      pv_l1 += std::fabs(v);
      const df d = df_from_double(v);
      pdf[(size_t)i] = make_float2(d.hi, d.lo);
    }
    // staged in gdf[1] (free before the solve starts), then relabelled
    GOPS_CUDA_TRY(cudaMemcpyAsync(g->ws.gdf[1], pdf.data(), sizeof(float2) * (size_t)n,
                                  cudaMemcpyHostToDevice, ctx->stream));
    permute_pdf<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div<int64_t>(n, 256), 4096)), 256, 0,
                  ctx->stream>>>(n, g->ws.gdf[1], g->perm, g->ws.pdf);
    GOPS_CUDA_TRY(cudaGetLastError());
    ctx->stats.h2d_bytes += sizeof(float2) * (size_t)n;
    ctx->stats.kernel_launches += 1;
    GOPS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (!std::isfinite(pv_l1)) pv_l1 = 1.0;
  }
  Status st;
  if (mode == kPlain) st = run_mode<kPlain>(ctx, g, cfg, pv_l1, run);
  else if (mode == kWeighted) st = run_mode<kWeighted>(ctx, g, cfg, pv_l1, run);
  else st = run_mode<kPpr>(ctx, g, cfg, pv_l1, run);
  GOPS_TRY(st);
  ctx->last_scores = g->ws.scores;
  if (scores_host) {
    GOPS_CUDA_TRY(cudaMemcpyAsync(scores_host, g->ws.scores, sizeof(double) * (size_t)g->n,
                                  cudaMemcpyDeviceToHost, ctx->stream));
    GOPS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    ctx->stats.d2h_bytes += sizeof(double) * (size_t)g->n;
  }
  return Status::ok();
}

}  // namespace gops
