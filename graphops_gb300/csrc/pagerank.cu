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
// Work layout.  Rows are relabelled by in-degree (descending) at build time,
// so each degree class is a contiguous segment.  A warp task covers 32/sw
// consecutive rows of one segment with sw lanes per row (sw chosen so a lane
// has about four edges); every lane keeps four independent column loads and
// four gathers in flight, and a row's sum is an xor-shuffle reduction over its
// sw lanes.  Rows above kHubThreshold in-edges are split into kHubChunk-edge
// warp tasks whose partials are combined, in chunk order, by the task that
// finishes last.  No block-wide barrier sits on the edge path.
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
// Iteration kernels: one 1024-thread block per SM (64 registers per thread
// fill the register file), and the first kGCache (hottest, after the
// in-degree relabelling) entries of the FP32 gathered vector staged in shared
// memory by every block of the weighted FP32 phase.  Measured at R-MAT 22: a
// 32 K-entry cache takes the weighted FP32 step from 0.246 to 0.231 ms; it
// does not pay for the unweighted step, nor for the double-float phase,
// whose 8-byte entries halve what fits.
constexpr int kIterThreads = 1024;
constexpr int kIterWarps = kIterThreads / kWarp;
constexpr int kGCache = 32768;
constexpr int kUnroll = 4;  // edges per lane per round and row (one 16-byte load)
// double-float phase while ||r||_1 >= kTheta.  Measured L1 against the FP64
// fixed point on R-MAT 16-20 (tol 1e-8): 4.5e-9 at 1e-2, 4.8e-9 at 3e-2,
// 6e-9 at 1e-1, for the same step counts; 1e-1 runs 3-4 fewer double-float
// steps (2.4 % of a solve at R-MAT 22) but leaves 2.7e-8 on a small dense
// random graph of the golden fixtures (bar 1e-8), so 1e-2 stays.
constexpr double kTheta = 1e-2;

struct IterParams {
  int64_t n;
  const int64_t *rp;
  const int32_t *col;
  const float *val;
  const float *deg;
  const uint32_t *dmask;
  const int32_t *hub_first;
  const int32_t *hub_task_row;
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
  __device__ static T zero() { return {0.0f, 0.0f}; }
  __device__ static T add(T a, T b) { return df_add(a, b); }
  __device__ static T shfl(T v, int m) { return shfl_xor_df(v, m, 32); }
  static constexpr bool kCache = false;
  template <int NC>
  __device__ static T load_g(const IterParams &p, const void *, int32_t u) {
    const float2 g = __ldg(&p.gdf_in[u]);
    return {g.x, g.y};
  }
  template <int NC>
  __device__ static void stage(const IterParams &, void *) {}
  __device__ static T scale(T g, float w) { return df_mul_f(g, w); }
  __device__ static float2 pack(T v) { return make_float2(v.hi, v.lo); }
  __device__ static T unpack(float2 v) { return {v.x, v.y}; }
};

struct PrecF32 {
  using T = float;
  static constexpr bool kDF = false;
  __device__ static T zero() { return 0.0f; }
  __device__ static T add(T a, T b) { return a + b; }
  __device__ static T shfl(T v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
  static constexpr bool kCache = true;
  // entries [0, NC) come from shared memory (u <= n: entries past n + 1 are
  // staged by no block and read by no edge)
  template <int NC>
  __device__ static T load_g(const IterParams &p, const void *cache, int32_t u) {
    if (NC > 0 && u < NC) return reinterpret_cast<const float *>(cache)[u];
    return __ldg(&p.gf_in[u]);
  }
  template <int NC>
  __device__ static void stage(const IterParams &p, void *cache) {
    float *c = reinterpret_cast<float *>(cache);
    const int lim = (int)(p.n + 1 < (int64_t)NC ? p.n + 1 : (int64_t)NC);  // entry n: padding
    for (int i = threadIdx.x; i < lim; i += blockDim.x) c[i] = __ldg(&p.gf_in[i]);
  }
  __device__ static T scale(T g, float w) { return g * w; }
  __device__ static float2 pack(T v) { return make_float2(v, 0.0f); }
  __device__ static T unpack(float2 v) { return v.x; }
};

// FP32 entries of the gathered vector staged in shared memory per block
template <class P, int MODE>
__host__ __device__ constexpr int cache_entries() {
  return P::kCache && MODE == kWeighted ? kGCache : 0;
}

struct Acc {
  long long l1 = 0, dang = 0;
  int bad = 0;
};

// Per-row inputs of the epilogue, loaded before the row's edges so their
// latency overlaps the edge loads: the running x part (acc in the
// double-float phase, tail in the FP32 phase), the out-degree, the dangling
// flag and the personalization entry.
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

// R rows per sub-warp, their edges interleaved so that every lane keeps
// R column loads (16 bytes: four edges each), then 4R gathers, in flight.
// Rows start and end on 4-edge boundaries (padding edges: column n, weight
// 0), so lane li of a row's sub-warp takes the quads li, li+SW, ... of each
// row and adds them in that order: a row's sum does not depend on R.
template <class P, int MODE, int R>
__device__ __forceinline__ void rows_sum(const IterParams &p, const void *cache,
                                         const int32_t (&eb)[R], const int32_t (&ee)[R], int li,
                                         int SW, typename P::T (&s)[R]) {
  static_assert(kRowAlign == 4 && kUnroll == 4, "one aligned quad per lane and round");
  constexpr int NC = cache_entries<P, MODE>();
  int32_t len = 0;
#pragma unroll
  for (int q = 0; q < R; ++q) {
    s[q] = P::zero();
    len = max(len, ee[q] - eb[q]);
  }
  for (int32_t off = 4 * li; off < len; off += 4 * SW) {
    int4 c[R];
    float4 w[R];
    bool ok[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const int32_t e = eb[q] + off;
      ok[q] = e < ee[q];
      c[q] = ok[q] ? __ldg(reinterpret_cast<const int4 *>(&p.col[e])) : make_int4(0, 0, 0, 0);
      w[q] = (MODE == kWeighted && ok[q]) ? __ldg(reinterpret_cast<const float4 *>(&p.val[e]))
                                          : make_float4(1.f, 1.f, 1.f, 1.f);
    }
    typename P::T g[R][4];
#pragma unroll
    for (int q = 0; q < R; ++q) {
      g[q][0] = ok[q] ? P::template load_g<NC>(p, cache, c[q].x) : P::zero();
      g[q][1] = ok[q] ? P::template load_g<NC>(p, cache, c[q].y) : P::zero();
      g[q][2] = ok[q] ? P::template load_g<NC>(p, cache, c[q].z) : P::zero();
      g[q][3] = ok[q] ? P::template load_g<NC>(p, cache, c[q].w) : P::zero();
    }
#pragma unroll
    for (int q = 0; q < R; ++q)
      if (ok[q]) {
        if (MODE == kWeighted) {
          s[q] = P::add(s[q], P::scale(g[q][0], w[q].x));
          s[q] = P::add(s[q], P::scale(g[q][1], w[q].y));
          s[q] = P::add(s[q], P::scale(g[q][2], w[q].z));
          s[q] = P::add(s[q], P::scale(g[q][3], w[q].w));
        } else {
          s[q] = P::add(s[q], g[q][0]);
          s[q] = P::add(s[q], g[q][1]);
          s[q] = P::add(s[q], g[q][2]);
          s[q] = P::add(s[q], g[q][3]);
        }
      }
  }
}

template <class P, int MODE>
__device__ __forceinline__ void row_task(const IterParams &p, const void *cache, const Segment &sg,
                                         int local, int lane, df dsum, Acc &a) {
  using T = typename P::T;
  constexpr int R = kRowsPerLane;
  const int SW = sg.sw;
  const int lg = 31 - __clz(SW);   // sw is a power of two
  const int RPW = 32 >> lg;        // rows per warp per interleave slot
  const int li = lane & (SW - 1);
  int64_t row[R];
  int32_t eb[R], ee[R];
  bool valid[R];
  RowIn in[R];
#pragma unroll
  for (int q = 0; q < R; ++q) {
    row[q] = (int64_t)sg.row_begin + ((int64_t)local * R + q) * RPW + (lane >> lg);
    valid[q] = row[q] < sg.row_end;
    eb[q] = valid[q] ? (int32_t)__ldg(&p.rp[row[q]]) : 0;
    ee[q] = valid[q] ? (int32_t)__ldg(&p.rp[row[q] + 1]) : 0;
  }
#pragma unroll
  for (int q = 0; q < R; ++q)
    if (valid[q] && li == 0) in[q] = row_in<P, MODE>(p, row[q]);
  T s[R];
  rows_sum<P, MODE, R>(p, cache, eb, ee, li, SW, s);
#pragma unroll
  for (int q = 0; q < R; ++q) {
    for (int o = SW >> 1; o > 0; o >>= 1) s[q] = P::add(s[q], P::shfl(s[q], o));
    if (valid[q] && li == 0) epilogue<P, MODE>(p, row[q], s[q], dsum, in[q], a);
  }
}

template <class P, int MODE>
__device__ __forceinline__ void hub_task(const IterParams &p, const void *cache, int t, int lane,
                                         df dsum, Acc &a) {
  using T = typename P::T;
  const int32_t h = __ldg(&p.hub_task_row[t]);
  const int32_t first = __ldg(&p.hub_first[h]);
  const int32_t nch = __ldg(&p.hub_first[h + 1]) - first;
  const int32_t rb = (int32_t)__ldg(&p.rp[h]), re = (int32_t)__ldg(&p.rp[h + 1]);
  const int32_t cs = rb + (t - first) * kHubChunk;
  const int32_t eb[1] = {cs}, ee[1] = {min(re, cs + kHubChunk)};
  T s[1];
  rows_sum<P, MODE, 1>(p, cache, eb, ee, lane, 32, s);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s[0] = P::add(s[0], P::shfl(s[0], o));
  if (lane == 0) {
    p.lpart[t] = P::pack(s[0]);
    __threadfence();
    const unsigned tk = atomicAdd(&p.lcnt[h], 1u);
    if (tk == (unsigned)(nch - 1)) {
      __threadfence();
      T sum = P::zero();
      for (int j = 0; j < nch; ++j) sum = P::add(sum, P::unpack(__ldcg(&p.lpart[first + j])));
      p.lcnt[h] = 0;
      const RowIn in = row_in<P, MODE>(p, h);
      epilogue<P, MODE>(p, h, sum, dsum, in, a);
    }
  }
}

template <class P, int MODE>
__global__ void __launch_bounds__(kIterThreads, 1) iterate_kernel(IterParams p) {
  __shared__ long long bred[2][kIterWarps];
  __shared__ int bbad[kIterWarps];
  extern __shared__ __align__(16) unsigned char gcache[];
  df dsum;
  if (!prologue<P::kDF>(p, &dsum)) return;
  if constexpr (P::kCache) {
    if (cache_entries<P, MODE>() > 0) {
      P::template stage<cache_entries<P, MODE>()>(p, gcache);
      __syncthreads();
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nwarps = gridDim.x * kIterWarps;
  Acc a;
  for (int t = blockIdx.x * kIterWarps + wid; t < p.plan.n_tasks; t += nwarps) {
    if (t < p.plan.n_hub_tasks) {
      hub_task<P, MODE>(p, gcache, t, lane, dsum, a);
      continue;
    }
    int si = 0;
    while (si + 1 < p.plan.n_segs && t >= p.plan.segs[si + 1].task_begin) ++si;
    const Segment sg = p.plan.segs[si];
    row_task<P, MODE>(p, gcache, sg, t - sg.task_begin, lane, dsum, a);
  }

  // ---- block totals of the exact fixed-point sums -> one atomic each
  long long l1 = warp_sum_ll(a.l1), dg = warp_sum_ll(a.dang);
  int bad = warp_or(a.bad);
  if (lane == 0) { bred[0][wid] = l1; bred[1][wid] = dg; bbad[wid] = bad; }
  __syncthreads();
  if (threadIdx.x == 0) {
    long long t1 = 0, t2 = 0;
    int tb = 0;
    for (int w = 0; w < kIterWarps; ++w) { t1 += bred[0][w]; t2 += bred[1][w]; tb |= bbad[w]; }
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
  cudaFree(ws.sums); cudaFree(ws.lpart); cudaFree(ws.lcnt); cudaFree(ws.state);
  ws = Workspace{};
}

Status workspace_alloc(Ctx *ctx, Graph *g);

// The solve workspace of a graph, allocated on first use; a failed
// allocation leaves none of it behind.
Status workspace_ensure(Ctx *ctx, Graph *g) {
  if (g->ws.sums) return Status::ok();
  Status st = workspace_alloc(ctx, g);
  if (st.code != GOPS_OK) {
    cudaStreamSynchronize(ctx->stream);
    workspace_free(g->ws);
  }
  return st;
}

Status workspace_alloc(Ctx *ctx, Graph *g) {
  Workspace &ws = g->ws;
  const size_t n = (size_t)std::max<int64_t>(g->n, 1);
  const size_t nht = (size_t)std::max<int32_t>(g->plan.n_hub_tasks, 1);
  const size_t nh = (size_t)std::max<int32_t>(g->plan.n_hub, 1);
  // one extra entry: index n is the column of row padding and always 0
  GOPS_CUDA_TRY(dev_malloc_async(&ws.gdf[0], sizeof(float2) * (n + 1), ctx->stream));
  GOPS_CUDA_TRY(dev_malloc_async(&ws.gdf[1], sizeof(float2) * (n + 1), ctx->stream));
  GOPS_CUDA_TRY(dev_malloc_async(&ws.gf[0], sizeof(float) * (n + 1), ctx->stream));
  GOPS_CUDA_TRY(dev_malloc_async(&ws.gf[1], sizeof(float) * (n + 1), ctx->stream));
  GOPS_CUDA_TRY(dev_malloc_async(&ws.acc, sizeof(float2) * n, ctx->stream));
  GOPS_CUDA_TRY(dev_malloc_async(&ws.tail, sizeof(float) * n, ctx->stream));
  GOPS_CUDA_TRY(dev_malloc_async(&ws.pdf, sizeof(float2) * n, ctx->stream));
  GOPS_CUDA_TRY(dev_malloc_async(&ws.scores, sizeof(double) * n, ctx->stream));
  GOPS_CUDA_TRY(dev_malloc_async(&ws.lpart, sizeof(float2) * nht, ctx->stream));
  GOPS_CUDA_TRY(dev_malloc_async(&ws.lcnt, sizeof(unsigned) * nh, ctx->stream));
  GOPS_CUDA_TRY(dev_malloc_async(&ws.state, sizeof(SolveState), ctx->stream));
  GOPS_CUDA_TRY(dev_malloc_async(&ws.sums, sizeof(long long) * 12, ctx->stream));
  ws.n = g->n;
  return Status::ok();
}

namespace {

template <class P, int MODE>
size_t iter_smem(const Graph *g) {
  return sizeof(float) * (size_t)std::min<int64_t>(g->n + 1, cache_entries<P, MODE>());
}

template <class P, int MODE>
int grid_for_iter(const Ctx *ctx, const Graph *g) {
  const size_t smem = iter_smem<P, MODE>(g);
  int occ = 0;
  if (smem > 0)
    cudaFuncSetAttribute(iterate_kernel<P, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, iterate_kernel<P, MODE>, kIterThreads, smem);
  occ = std::max(1, occ);
  const int64_t blocks_needed = ceil_div<int64_t>(std::max<int32_t>(g->plan.n_tasks, 1), kIterWarps);
  return (int)std::max<int64_t>(1, std::min<int64_t>(blocks_needed, (int64_t)ctx->num_sms * occ));
}

template <int MODE>
Status run_mode(Ctx *ctx, Graph *g, Workspace &ws, const gops_config *cfg, double pv_l1,
                gops_run *run) {
  cudaStream_t s = ctx->stream;
  IterParams p{};
  p.n = g->n;
  p.rp = g->in_rp;
  p.col = g->in_col;
  p.val = g->in_val;
  p.deg = g->deg;
  p.dmask = g->dmask_w;
  p.hub_first = g->hub_first;
  p.hub_task_row = g->hub_task_row;
  p.plan = g->plan;
  p.acc = ws.acc;
  p.tail = ws.tail;
  p.pdf = ws.pdf;
  p.sums = ws.sums;
  p.st = ws.state;
  p.lpart = ws.lpart;
  p.lcnt = ws.lcnt;
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
  for (int b = 0; b < 2; ++b) {  // padding entry n of the gathered vectors
    GOPS_CUDA_TRY(cudaMemsetAsync(ws.gdf[b] + g->n, 0, sizeof(float2), s));
    GOPS_CUDA_TRY(cudaMemsetAsync(ws.gf[b] + g->n, 0, sizeof(float), s));
  }
  GOPS_CUDA_TRY(cudaMemsetAsync(ws.state, 0, sizeof(SolveState), s));
  GOPS_CUDA_TRY(cudaMemsetAsync(ws.lcnt, 0, sizeof(unsigned) * std::max<int32_t>(g->plan.n_hub, 1), s));
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

  const int grid_df = grid_for_iter<PrecDF, MODE>(ctx, g);
  const int grid_f = grid_for_iter<PrecF32, MODE>(ctx, g);
  const size_t smem_df = iter_smem<PrecDF, MODE>(g), smem_f = iter_smem<PrecF32, MODE>(g);
  bool f32_known = false;
  unsigned long long k = 1;
  const int chunk = 4;
  // per-launch timing: (step, is_df) of every timed launch, events 2i / 2i+1
  std::vector<std::pair<unsigned long long, bool>> timed;
  auto timed_launch = [&](bool is_df) -> Status {
    if (!ctx->timing) return Status::ok();
    const size_t need = 2 * (timed.size() + 1);
    while (ctx->tev.size() < need) {
      cudaEvent_t e;
      GOPS_CUDA_TRY(cudaEventCreate(&e));
      ctx->tev.push_back(e);
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
        iterate_kernel<PrecDF, MODE><<<grid_df, kIterThreads, smem_df, s>>>(p);
        if (ctx->timing) GOPS_CUDA_TRY(cudaEventRecord(ctx->tev[2 * timed.size() - 1], s));
        ++launches;
      }
      if (k >= 2) {
        GOPS_TRY(timed_launch(false));
        if (ctx->timing) GOPS_CUDA_TRY(cudaEventRecord(ctx->tev[2 * timed.size() - 2], s));
        iterate_kernel<PrecF32, MODE><<<grid_f, kIterThreads, smem_f, s>>>(p);
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
  GOPS_CUDA_TRY(cudaEventRecord(ctx->ev[2], s));
  finalize_kernel<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div<int64_t>(g->n, 256), 4096)),
                    256, 0, s>>>(g->n, ws.acc, ws.tail, g->perm, ws.scores);
  GOPS_CUDA_TRY(cudaGetLastError());
  ++launches;
  GOPS_CUDA_TRY(cudaEventRecord(ctx->ev[3], s));
  GOPS_CUDA_TRY(cudaEventSynchronize(ctx->ev[3]));
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
      const bool active = kk <= its && (is_df ? (f32_from == 0 || kk < f32_from) : (f32_from && kk >= f32_from));
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
  if (mode == kPlain) st = run_mode<kPlain>(ctx, g, g->ws, cfg, pv_l1, run);
  else if (mode == kWeighted) st = run_mode<kWeighted>(ctx, g, g->ws, cfg, pv_l1, run);
  else st = run_mode<kPpr>(ctx, g, g->ws, cfg, pv_l1, run);
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

// Plain PageRank (as solve(.., kPlain, ..)) on a workspace the caller
// provides; performs no device or pinned allocation of its own.
Status solve_plain_in_workspace(Ctx *ctx, Graph *g, const gops_config *cfg, Workspace &ws,
                                double *scores_host, gops_run *run) {
  ctx->stats = gops_stats{};
  if (g->n == 0) {
    run->iterations = 0;
    run->diff_l1 = 0.0;
    run->converged = 1;
    run->reserved = 0;
    return Status::ok();
  }
  const bool timing = ctx->timing;
  ctx->timing = false;  // per-launch timing would create events
  Status st = run_mode<kPlain>(ctx, g, ws, cfg, 1.0, run);
  ctx->timing = timing;
  GOPS_TRY(st);
  ctx->last_scores = ws.scores;
  if (scores_host) {
    GOPS_CUDA_TRY(cudaMemcpyAsync(scores_host, ws.scores, sizeof(double) * (size_t)g->n,
                                  cudaMemcpyDeviceToHost, ctx->stream));
    GOPS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    ctx->stats.d2h_bytes += sizeof(double) * (size_t)g->n;
  }
  return Status::ok();
}

}  // namespace gops
