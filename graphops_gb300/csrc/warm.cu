// The learned warm start for batched personalized PageRank (include/gops.h,
// gops_warm_*): graph-side state, the exact sparse push, the least-squares
// cluster coupling, the loss, and the train / predict / solve drivers.  The
// network itself is in warm_nn.cu.
//
// For a seed set with normalised indicator s, damping d and transition P:
//   x0 = (1-d)(s + d P s + d^2 P^2 s + d^3 P^3 s)        push, exact
//      + tm * w_i * m[a_i] / (sum_c m_c * cw[a_i])       learned tail
// tm = 1 - mass of the exact part; a_i = k-means cluster of node i over the
// random-projection code; m = relu(c K) with c = [cluster mix of P^3 s,
// cluster mix of P^4 s, 1]; w = exp(MPNN); cw[c] = sum of w over cluster c.
// Every sum that decides a result is either integer (fixed point) or taken
// in a fixed order, so predictions and training are bit-reproducible.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "primitives.cuh"
#include "warm.cuh"

namespace gops {

Status ppr_batch(Ctx *ctx, Graph *g, const gops_config *cfg, int64_t nsets, const int64_t *seed_ptr,
                 const int32_t *seed_idx, const float *x0, bool x0_on_device, float *scores,
                 bool scores_on_device, gops_run *runs, const double *r1_max, int32_t *rejected);

namespace {

using bf16 = __nv_bfloat16;

constexpr int kPushThreads = 512;
constexpr int kMaxSeeds = 1024;  // distinct seeds of a set handled by the push
constexpr int kMaxL1 = 2048;     // out-edges of a set's seeds handled by the push
constexpr float kFixF = 1099511627776.0f;  // 2^40 (kWFix)

// A 2^40 fixed-point value as FP32: one rounding (64-bit integer to FP32),
// then an exact power-of-two scale; the same value as (float)(f / 2^40) in
// FP64 without FP64 instructions (issued at a small fraction of the FP32 rate
// on this GPU).
__device__ __forceinline__ float fix40_to_float(long long f) { return __ll2float_rn(f) * (1.0f / kFixF); }
constexpr double kCentFix = 1073741824.0;  // 2^30: fixed point of the k-means sums
constexpr int kKmeansRestarts = 8;        // k-means runs per model; the lowest within-cluster sum is kept

__host__ __device__ inline uint64_t mix64(uint64_t z) {  // SplitMix64 (Steele, Lea, Flood 2014)
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ long long fx40(float v) { return __float2ll_rn(v * kFixF); }

// ---------------------------------------------------------------------------
// graph-side state
// ---------------------------------------------------------------------------
__global__ void expand_src(const int64_t *rp, int64_t n, uint32_t *src) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t u = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); u < n; u += nw)
    for (int64_t e = rp[u] + lane; e < rp[u + 1]; e += 32) src[e] = (uint32_t)u;
}

__global__ void copy_keys(const int32_t *col, int64_t m, uint32_t *keys) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x)
    keys[e] = (uint32_t)col[e];
}

// rp[v] = first position whose key >= v (keys sorted), rp[n] = m
__global__ void offsets_from_sorted(const uint32_t *keys, int64_t m, int64_t n, int64_t *rp) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= m; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t prev = i == 0 ? -1 : (int64_t)keys[i - 1];
    const int64_t cur = i == m ? n : (int64_t)keys[i];
    for (int64_t v = prev + 1; v <= cur; ++v) rp[v] = i;
  }
}

__global__ void degree_terms(const int64_t *out_rp, const int64_t *in_rp, int64_t n, float *inv_out, float *inv_in) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t dout = out_rp[i + 1] - out_rp[i], din = in_rp[i + 1] - in_rp[i];
    inv_out[i] = dout > 0 ? 1.0f / (float)dout : 0.0f;
    inv_in[i] = din > 0 ? 1.0f / (float)din : 0.0f;
  }
}

// Cluster distributions of out-neighbourhoods as sparse runs:
//   LEVEL 1: h(w)[c]  = #{x in out(w): a_x = c} / deg(w)
//   LEVEL 2: h2(w)[c] = sum over x in out(w) of h(x)[c] / deg(w)
// A warp per node sums its bins in a warp-private fixed-point histogram
// (order-independent); the count pass writes the number of nonzero bins,
// the fill pass writes them in cluster order at rp[w].
template <int LEVEL>
__global__ void runs_kernel(const int64_t *out_rp, const int32_t *out_col, const float *inv_out,
                            const int32_t *cluster, const int64_t *hrp, const int32_t *hcl, const float *hwt,
                            int64_t n, int r, int64_t *rp, int32_t *ocl, float *owt, int fill) {
  extern __shared__ __align__(16) long long hsm[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  long long *h = hsm + (int64_t)wid * r;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + wid; w < n; w += nw) {
    for (int c = lane; c < r; c += 32) h[c] = 0;
    __syncwarp();
    const float iw = inv_out[w];
    for (int64_t e = out_rp[w] + lane; e < out_rp[w + 1]; e += 32) {
      const int32_t x = out_col[e];
      if (LEVEL == 1) {
        atomicAdd(reinterpret_cast<unsigned long long *>(&h[cluster[x]]), (unsigned long long)fx40(iw));
      } else {
        for (int64_t q = hrp[x]; q < hrp[x + 1]; ++q)
          atomicAdd(reinterpret_cast<unsigned long long *>(&h[hcl[q]]), (unsigned long long)fx40(hwt[q] * iw));
      }
    }
    __syncwarp();
    if (!fill) {
      int cnt = 0;
      for (int c = lane; c < r; c += 32) cnt += h[c] != 0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
      if (lane == 0) rp[w] = cnt;
    } else {
      int64_t base = rp[w];
      for (int c0 = 0; c0 < r; c0 += 32) {
        const int c = c0 + lane;
        const bool nz = c < r && h[c] != 0;
        const unsigned mask = __ballot_sync(0xffffffffu, nz);
        if (nz) {
          const int64_t pos = base + __popc(mask & ((1u << lane) - 1u));
          ocl[pos] = c;
          owt[pos] = fix40_to_float((long long)h[c]);
        }
        base += __popc(mask);
      }
    }
    __syncwarp();
  }
}

// standard normal entries from a counter-based generator: two 24-bit
// uniforms per entry, Box-Muller transform
__global__ void code_init(int64_t count, uint64_t seed, float *z) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t h = mix64(seed ^ mix64((uint64_t)i));
    const float u1 = (float)((h >> 40) + 1) * (1.0f / 16777216.0f);
    const float u2 = (float)((h >> 16) & 0xFFFFFFull) * (1.0f / 16777216.0f);
    z[i] = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
  }
}

// one diffusion step of the code: out = (mean over in-neighbours + mean over
// out-neighbours) / 2; a half-warp per node, a lane per code column
__global__ void code_step(const int64_t *in_rp, const int32_t *in_col, const float *inv_in, const int64_t *out_rp,
                          const int32_t *out_col, const float *inv_out, const float *z, int64_t n, float *out) {
  const int k = threadIdx.x & 15;
  const int64_t nh = (int64_t)gridDim.x * (blockDim.x >> 4);
  for (int64_t v = (int64_t)blockIdx.x * (blockDim.x >> 4) + (threadIdx.x >> 4); v < n; v += nh) {
    float a = 0.f, b = 0.f;
    for (int64_t e = in_rp[v]; e < in_rp[v + 1]; ++e) a += z[(int64_t)in_col[e] * kWCode + k];
    for (int64_t e = out_rp[v]; e < out_rp[v + 1]; ++e) b += z[(int64_t)out_col[e] * kWCode + k];
    out[v * kWCode + k] = 0.5f * (a * inv_in[v] + b * inv_out[v]);
  }
}

// out[v][0..C) = inv_in[v] * sum over in-edges of in[u][0..C) (warp per node)
__global__ void agg_small(const int64_t *in_rp, const int32_t *in_col, const float *inv_in, const float *in, int C,
                          int64_t n, float *out, int ldo) {
  const int k = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t v = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); v < n; v += nw) {
    if (k >= C) continue;
    float a = 0.f;
    for (int64_t e = in_rp[v]; e < in_rp[v + 1]; ++e) a += in[(int64_t)in_col[e] * C + k];
    out[v * ldo + k] = a * inv_in[v];
  }
}

// per-block column sums and sums of squares of a row-major n x C matrix
// (C divides the block size), FP64 partials in a fixed order
__global__ void col_stats(const float *a, int64_t n, int C, double *part) {
  __shared__ double ss[256], sq[256];
  const int64_t total = n * C;
  double s = 0.0, q = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = a[i];
    s += v;
    q += v * v;
  }
  ss[threadIdx.x] = s;
  sq[threadIdx.x] = q;
  __syncthreads();
  if ((int)threadIdx.x < C) {
    double ts = 0.0, tq = 0.0;
    for (int t = threadIdx.x; t < (int)blockDim.x; t += C) {
      ts += ss[t];
      tq += sq[t];
    }
    part[(int64_t)blockIdx.x * 2 * C + threadIdx.x] = ts;
    part[(int64_t)blockIdx.x * 2 * C + C + threadIdx.x] = tq;
  }
}

__global__ void col_apply(float *a, int64_t n, int C, const float *mean, const float *inv_sd) {
  const int64_t total = n * C;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(i % C);
    a[i] = (a[i] - mean[k]) * inv_sd[k];
  }
}

__global__ void base_features(const int64_t *out_rp, const int64_t *in_rp, const float *code, int64_t n, float *x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i * kWFeat + 0] = log1pf((float)(out_rp[i + 1] - out_rp[i]));
    x[i * kWFeat + 1] = log1pf((float)(in_rp[i + 1] - in_rp[i]));
    for (int k = 0; k < kWCode; ++k) x[i * kWFeat + 2 + k] = code[i * kWCode + k];
  }
}

__global__ void pack_x1(const float *x, const float *ax, int64_t n, bf16 *x1) {
  const int64_t total = n * kWIn;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = i / kWIn;
    const int k = (int)(i % kWIn);
    float val = 0.f;
    if (k < kWFeat) val = x[v * kWFeat + k];
    else if (k < 2 * kWFeat) val = ax[v * kWFeat + (k - kWFeat)];
    else if (k == kWBiasCol) val = 1.f;
    x1[i] = __float2bfloat16_rn(val);
  }
}

__global__ void pack_y(const float *code, const float *acode, int64_t n, float *y) {
  const int64_t total = n * kWY;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = i / kWY;
    const int k = (int)(i % kWY);
    y[i] = k < kWCode ? code[v * kWCode + k] : acode[v * kWCode + (k - kWCode)];
  }
}

// t3[u][:] = sum over v in out(u) of h2(v)[:] / deg(u): a warp per node,
// fixed-point sums in a warp-private histogram, written as a dense row
__global__ void table_from_runs(const int64_t *out_rp, const int32_t *out_col, const float *inv_out,
                                const int64_t *hrp, const int32_t *hcl, const float *hwt, int64_t n, int r,
                                float *T) {
  extern __shared__ __align__(16) long long tsm[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  long long *h = tsm + (int64_t)wid * r;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t u = (int64_t)blockIdx.x * (blockDim.x >> 5) + wid; u < n; u += nw) {
    for (int c = lane; c < r; c += 32) h[c] = 0;
    __syncwarp();
    const float iu = inv_out[u];
    for (int64_t e = out_rp[u] + lane; e < out_rp[u + 1]; e += 32) {
      const int32_t v = out_col[e];
      for (int64_t q = hrp[v]; q < hrp[v + 1]; ++q)
        atomicAdd(reinterpret_cast<unsigned long long *>(&h[hcl[q]]), (unsigned long long)fx40(hwt[q] * iu));
    }
    __syncwarp();
    for (int c = lane; c < r; c += 32) T[u * r + c] = fix40_to_float((long long)h[c]);
    __syncwarp();
  }
}

// t4[u][:] = sum over v in out(u) of t3[v][:] / deg(u): a warp per node,
// lanes over bins, out-edges in order
__global__ void table_next(const int64_t *out_rp, const int32_t *out_col, const float *inv_out, const float *T3,
                           int64_t n, int r, float *T4) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t u = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); u < n; u += nw) {
    float acc[kWMaxClusters / 32];
#pragma unroll
    for (int k = 0; k < kWMaxClusters / 32; ++k) acc[k] = 0.f;
    for (int64_t e = out_rp[u]; e < out_rp[u + 1]; ++e) {
      const int64_t v = out_col[e];
#pragma unroll
      for (int k = 0; k < kWMaxClusters / 32; ++k)
        if (lane + 32 * k < r) acc[k] += T3[v * r + lane + 32 * k];
    }
    const float iu = inv_out[u];
#pragma unroll
    for (int k = 0; k < kWMaxClusters / 32; ++k)
      if (lane + 32 * k < r) T4[u * r + lane + 32 * k] = acc[k] * iu;
  }
}

// ---- k-means (k-means++ seeding, Arthur & Vassilvitskii 2007; Lloyd iterations)
__global__ void kmpp_dist(const float *y, int64_t n, const float *c, int first, float *d2) {
  __shared__ float cs[kWY];
  if (threadIdx.x < kWY) cs[threadIdx.x] = c[threadIdx.x];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int k = 0; k < kWY; ++k) {
      const float t = y[i * kWY + k] - cs[k];
      s = fmaf(t, t, s);
    }
    d2[i] = first ? s : fminf(d2[i], s);
  }
}

constexpr int kChunk = 1024;
__global__ void chunk_sums(const float *d2, int64_t n, double *out) {
  __shared__ double sh[256];
  const int64_t base = (int64_t)blockIdx.x * kChunk;
  double s = 0.0;
  for (int j = 0; j < kChunk / 256; ++j) {
    const int64_t i = base + threadIdx.x * (kChunk / 256) + j;
    if (i < n) s += (double)d2[i];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

__global__ void km_assign(const float *y, int64_t n, const float *cent, int r, int32_t *a, long long *sums,
                          int *counts, float *best_d2) {
  extern __shared__ __align__(16) unsigned char sm[];
  float *cs = reinterpret_cast<float *>(sm);                             // r x kWY
  long long *acc = reinterpret_cast<long long *>(cs + r * kWY);          // r x kWY
  int *cnt = reinterpret_cast<int *>(acc + r * kWY);                     // r
  for (int i = threadIdx.x; i < r * kWY; i += blockDim.x) {
    cs[i] = cent[i];
    acc[i] = 0;
  }
  for (int i = threadIdx.x; i < r; i += blockDim.x) cnt[i] = 0;
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float yi[kWY];
#pragma unroll
    for (int k = 0; k < kWY; ++k) yi[k] = y[i * kWY + k];
    float best = INFINITY;
    int bc = 0;
    for (int c = 0; c < r; ++c) {
      float s = 0.f;
#pragma unroll
      for (int k = 0; k < kWY; ++k) {
        const float t = yi[k] - cs[c * kWY + k];
        s = fmaf(t, t, s);
      }
      if (s < best) {
        best = s;
        bc = c;
      }
    }
    a[i] = bc;
    if (best_d2) best_d2[i] = best;
    if (sums) {
#pragma unroll
      for (int k = 0; k < kWY; ++k)
        atomicAdd(reinterpret_cast<unsigned long long *>(&acc[bc * kWY + k]),
                  (unsigned long long)__double2ll_rn((double)yi[k] * kCentFix));
      atomicAdd(&cnt[bc], 1);
    }
  }
  if (!sums) return;
  __syncthreads();
  for (int i = threadIdx.x; i < r * kWY; i += blockDim.x)
    if (acc[i]) atomicAdd(reinterpret_cast<unsigned long long *>(&sums[i]), (unsigned long long)acc[i]);
  for (int i = threadIdx.x; i < r; i += blockDim.x)
    if (cnt[i]) atomicAdd(&counts[i], cnt[i]);
}

__global__ void km_update(float *cent, int r, long long *sums, int *counts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= r * kWY) return;
  const int c = i / kWY;
  if (counts[c] > 0) cent[i] = (float)((double)sums[i] / kCentFix / (double)counts[c]);
}

__global__ void iota_u32(uint32_t *v, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] = (uint32_t)i;
}

// ---------------------------------------------------------------------------
// the push: exact local terms, cluster mixes, tail mass and cold residual
// ---------------------------------------------------------------------------
struct PushArgs {
  const int64_t *out_rp;
  const int32_t *out_col;
  const float *inv_out;
  const float *t3, *t4;  // per-node cluster distributions of P^3 e_u and P^4 e_u
  const int32_t *cluster;
  const int64_t *sptr;  // set offsets into sidx (device)
  const int32_t *sidx;
  int64_t n;
  int r;
  float d;
  int64_t budget;
  long long *push;  // set-major, n per set (fixed point 2^40)
  double *mix;      // 2r + 1 per set
  double *tmass;
  double *r1c;
  int32_t *over;
};

__device__ int upper_bound_i64(const int64_t *a, int len, int64_t key) {  // first index with a[i] > key
  int lo = 0, hi = len;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] <= key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__device__ int find_sorted(const int32_t *a, int len, int32_t key) {  // index of key or -1
  int lo = 0, hi = len;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo < len && a[lo] == key ? lo : -1;
}

// block-wide inclusive scan of v (kPushThreads threads); returns the total
__device__ int64_t block_scan(int64_t *v, int len, int64_t *tmp) {
  // sequential over chunks of the block size: each thread scans its slice
  const int per = (len + kPushThreads - 1) / kPushThreads;
  const int b = threadIdx.x * per, e = min(len, b + per);
  int64_t s = 0;
  for (int i = b; i < e; ++i) {
    s += v[i];
    v[i] = s;
  }
  tmp[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t run = 0;
    for (int t = 0; t < kPushThreads; ++t) {
      const int64_t x = tmp[t];
      tmp[t] = run;
      run += x;
    }
    tmp[kPushThreads] = run;
  }
  __syncthreads();
  const int64_t off = tmp[threadIdx.x];
  for (int i = b; i < e; ++i) v[i] += off;
  __syncthreads();
  const int64_t total = tmp[kPushThreads];
  __syncthreads();
  return total;
}

struct PushSmem {
  int32_t seeds[kMaxSeeds];      // distinct seeds, sorted
  int32_t scount[kMaxSeeds];     // occurrences of each
  long long f1s[kMaxSeeds];      // (P s) at each seed, fixed point
  int64_t pre0[kMaxSeeds];       // inclusive prefix of seed out-degrees
  int32_t l1node[kMaxL1];        // level-1 items (out-edges of the seeds)
  float l1a[kMaxL1];             //   their mass
  float l1iv[kMaxL1];            //   1 / out-degree of the item's node
  int64_t l1rp[kMaxL1];          //   first out-edge of the item's node
  int64_t pre1[kMaxL1];          // inclusive prefix of level-1 out-degrees
  long long mass[4];
  int64_t tmp[kPushThreads + 1];
  int nseeds, over;
};

__global__ void __launch_bounds__(kPushThreads, 2) push_kernel(PushArgs p) {
  extern __shared__ __align__(16) unsigned char smraw[];
  PushSmem &S = *reinterpret_cast<PushSmem *>(smraw);
  const int64_t set = blockIdx.x;
  const int64_t a0 = p.sptr[set], a1 = p.sptr[set + 1];
  const int64_t L = a1 - a0;
  long long *loc = p.push + set * p.n;
  const float ws = L > 0 ? 1.0f / (float)L : 0.f;
  const float d = p.d, omd = 1.0f - p.d;
  if (threadIdx.x == 0) {
    S.over = L == 0 ? 2 : 0;  // 2: empty set (uniform personalization)
    S.nseeds = 0;
  }
  if (threadIdx.x < 4) S.mass[threadIdx.x] = 0;
  __syncthreads();
  // distinct sorted seeds with counts (a single thread: at most kMaxSeeds)
  if (threadIdx.x == 0 && S.over == 0) {
    if (L > 4 * kMaxSeeds) {
      S.over = 1;
    } else {
      int ns = 0;
      for (int64_t k = a0; k < a1 && ns <= kMaxSeeds; ++k) {
        const int32_t u = p.sidx[k];
        // insertion into the sorted distinct list
        int pos = ns;
        while (pos > 0 && S.seeds[pos - 1] > u) --pos;
        if (pos > 0 && S.seeds[pos - 1] == u) {
          ++S.scount[pos - 1];
          continue;
        }
        if (ns == kMaxSeeds) {
          ns = kMaxSeeds + 1;
          break;
        }
        for (int q = ns; q > pos; --q) {
          S.seeds[q] = S.seeds[q - 1];
          S.scount[q] = S.scount[q - 1];
        }
        S.seeds[pos] = u;
        S.scount[pos] = 1;
        ++ns;
      }
      if (ns > kMaxSeeds) S.over = 1;
      else S.nseeds = ns;
    }
  }
  __syncthreads();
  const int ns = S.nseeds;
  // seed out-degrees -> level-1 item count
  for (int i = threadIdx.x; i < ns; i += blockDim.x) {
    const int32_t u = S.seeds[i];
    S.pre0[i] = p.out_rp[u + 1] - p.out_rp[u];
    S.f1s[i] = 0;
  }
  __syncthreads();
  int64_t L1 = 0;
  if (S.over == 0) L1 = block_scan(S.pre0, ns, S.tmp);
  if (threadIdx.x == 0 && S.over == 0 && L1 > kMaxL1) S.over = 1;
  __syncthreads();
  // level-1 items: (v, alpha1 = s_u / deg(u)), with the degree of v
  if (S.over == 0)
    for (int t = threadIdx.x; t < (int)L1; t += blockDim.x) {
      const int i = upper_bound_i64(S.pre0, ns, t);
      const int32_t u = S.seeds[i];
      const int64_t first = i == 0 ? 0 : S.pre0[i - 1];
      const int32_t v = __ldg(&p.out_col[__ldg(&p.out_rp[u]) + (t - first)]);
      const int64_t rb = __ldg(&p.out_rp[v]), re = __ldg(&p.out_rp[v + 1]);
      S.l1node[t] = v;
      S.l1a[t] = (ws * (float)S.scount[i]) * __ldg(&p.inv_out[u]);
      S.l1iv[t] = __ldg(&p.inv_out[v]);
      S.l1rp[t] = rb;
      S.pre1[t] = re - rb;
    }
  __syncthreads();
  int64_t L2 = 0;
  if (S.over == 0) L2 = block_scan(S.pre1, (int)L1, S.tmp);
  if (threadIdx.x == 0 && S.over == 0 && L2 > p.budget) S.over = 1;
  __syncthreads();
  // visits of the level-3 and level-4 loops, against the budget
  if (S.over == 0) {
    int64_t work = 0;
    for (int64_t t = threadIdx.x; t < L2; t += blockDim.x) {
      const int i = upper_bound_i64(S.pre1, (int)L1, t);
      const int64_t first = i == 0 ? 0 : S.pre1[i - 1];
      const int32_t w = __ldg(&p.out_col[S.l1rp[i] + (t - first)]);
      work += __ldg(&p.out_rp[w + 1]) - __ldg(&p.out_rp[w]);
    }
    S.tmp[threadIdx.x] = work;
    __syncthreads();
    if (threadIdx.x == 0) {
      int64_t tot = L2;
      for (int t = 0; t < kPushThreads; ++t) tot += S.tmp[t];
      if (tot > p.budget) S.over = 1;
    }
    __syncthreads();
  }
  const int over = S.over;
  if (over) {
    // cold start: x0 = s (the empty set is handled by the composer)
    if (over == 1)
      for (int64_t k = a0 + threadIdx.x; k < a1; k += blockDim.x)
        atomicAdd(reinterpret_cast<unsigned long long *>(&loc[p.sidx[k]]), (unsigned long long)fx40(ws));
    for (int i = threadIdx.x; i < 2 * p.r + 1; i += blockDim.x) p.mix[set * (2 * p.r + 1) + i] = 0.0;
    if (threadIdx.x == 0) {
      p.tmass[set] = 0.0;
      p.r1c[set] = INFINITY;
      p.over[set] = over;
    }
    return;
  }
  // hop 0
  for (int i = threadIdx.x; i < ns; i += blockDim.x) {
    const float si = ws * (float)S.scount[i];
    atomicAdd(reinterpret_cast<unsigned long long *>(&loc[S.seeds[i]]), (unsigned long long)fx40(omd * si));
    if (p.out_rp[S.seeds[i] + 1] > p.out_rp[S.seeds[i]])
      atomicAdd(reinterpret_cast<unsigned long long *>(&S.mass[1]), (unsigned long long)fx40(si));
  }
  // hop 1 (and P s at the seeds, for the cold residual)
  const float c1 = omd * d, c2 = c1 * d, c3 = c2 * d;
  for (int t = threadIdx.x; t < (int)L1; t += blockDim.x) {
    const int32_t v = S.l1node[t];
    const float a = S.l1a[t];
    atomicAdd(reinterpret_cast<unsigned long long *>(&loc[v]), (unsigned long long)fx40(c1 * a));
    if (p.inv_out[v] > 0.f) atomicAdd(reinterpret_cast<unsigned long long *>(&S.mass[2]), (unsigned long long)fx40(a));
    const int si = find_sorted(S.seeds, ns, v);
    if (si >= 0) atomicAdd(reinterpret_cast<unsigned long long *>(&S.f1s[si]), (unsigned long long)fx40(a));
  }
  // hops 2 and 3; each item's loads are issued together (one dependent round
  // trip for w, one for its range, then its out-edges four at a time)
  long long m3 = 0;
  for (int64_t t = threadIdx.x; t < L2; t += blockDim.x) {
    const int i = upper_bound_i64(S.pre1, (int)L1, t);
    const int64_t first = i == 0 ? 0 : S.pre1[i - 1];
    const int32_t w = __ldg(&p.out_col[S.l1rp[i] + (t - first)]);
    const float a2 = S.l1a[i] * S.l1iv[i];
    const float iw = __ldg(&p.inv_out[w]);
    const int64_t eb = __ldg(&p.out_rp[w]), ee = __ldg(&p.out_rp[w + 1]);
    atomicAdd(reinterpret_cast<unsigned long long *>(&loc[w]), (unsigned long long)fx40(c2 * a2));
    if (iw == 0.f) continue;
    m3 += fx40(a2);
    const unsigned long long a3c = (unsigned long long)fx40(c3 * (a2 * iw));
    int64_t e = eb;
    for (; e + 4 <= ee; e += 4) {
      const int32_t x0 = __ldg(&p.out_col[e]), x1 = __ldg(&p.out_col[e + 1]);
      const int32_t x2 = __ldg(&p.out_col[e + 2]), x3 = __ldg(&p.out_col[e + 3]);
      atomicAdd(reinterpret_cast<unsigned long long *>(&loc[x0]), a3c);
      atomicAdd(reinterpret_cast<unsigned long long *>(&loc[x1]), a3c);
      atomicAdd(reinterpret_cast<unsigned long long *>(&loc[x2]), a3c);
      atomicAdd(reinterpret_cast<unsigned long long *>(&loc[x3]), a3c);
    }
    for (; e < ee; ++e) atomicAdd(reinterpret_cast<unsigned long long *>(&loc[__ldg(&p.out_col[e])]), a3c);
  }
  S.tmp[threadIdx.x] = m3;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long t3 = 0;
    for (int q = 0; q < kPushThreads; ++q) t3 += S.tmp[q];
    S.mass[3] = t3;
  }
  __syncthreads();
  // cluster mixes of P^3 s and P^4 s: the seeds' rows of t3 and t4 weighted
  // by their share of s (linear in s), summed in seed order
  const int F = 2 * p.r + 1;
  for (int i = threadIdx.x; i < 2 * p.r; i += blockDim.x) {
    const float *T = i < p.r ? p.t3 : p.t4;
    const int c = i < p.r ? i : i - p.r;
    double acc = 0.0;
    for (int k = 0; k < ns; ++k)
      acc += (double)(ws * (float)S.scount[k]) * (double)__ldg(&T[(int64_t)S.seeds[k] * p.r + c]);
    p.mix[set * F + i] = acc;
  }
  if (threadIdx.x == 0) {
    p.mix[set * F + 2 * p.r] = 1.0;
    // mass[1..3]: non-dangling mass of hops 0..2 = total mass of hops 1..3
    const double m1 = (double)S.mass[1] / kWFix, m2 = (double)S.mass[2] / kWFix, m3 = (double)S.mass[3] / kWFix;
    const double dd = (double)d;
    p.tmass[set] = 1.0 - (1.0 - dd) * (1.0 + dd * m1 + dd * dd * m2 + dd * dd * dd * m3);
    // ||F(s) - s||_1 = d * sum_v |P s (v) - (1 - D) s(v)|, D = dangling seed mass
    //               = d * (2 (1 - D) - 2 sum_seeds min(P s (v), (1 - D) s(v)))
    double mn = 0.0;
    for (int i = 0; i < ns; ++i)
      mn += fmin((double)S.f1s[i] / kWFix, m1 * (double)(ws * (float)S.scount[i]));
    p.r1c[set] = dd * (2.0 * m1 - 2.0 * mn);
    p.over[set] = 0;
  }
}

// coef[j][c] = tm_j * m_jc / (sum_c m_jc * cw_c), m = relu(mix_j K); zero for cold sets
__global__ void coef_kernel(const double *mix, const float *K, const float *cw, const double *tmass,
                            const int32_t *over, int r, float *coef) {
  __shared__ double xs[2 * kWMaxClusters + 1];
  __shared__ float red[kWMaxClusters];
  const int j = blockIdx.x, F = 2 * r + 1;
  for (int f = threadIdx.x; f < F; f += blockDim.x) xs[f] = mix[(int64_t)j * F + f];
  __syncthreads();
  float mc = 0.f;
  if ((int)threadIdx.x < r) {
    double s = 0.0;
    for (int f = 0; f < F; ++f) s += xs[f] * (double)K[(int64_t)f * r + threadIdx.x];
    mc = s > 0.0 ? (float)s : 0.f;
    red[threadIdx.x] = mc;
  }
  __syncthreads();
  if ((int)threadIdx.x < r) {
    float tot = 0.f;
    for (int c = 0; c < r; ++c) tot += red[c];  // fixed order
    const float c_w = cw[threadIdx.x];
    const bool ok = over[j] == 0 && tot > 0.f && c_w > 0.f;
    coef[(int64_t)j * r + threadIdx.x] = ok ? (float)tmass[j] * mc / (tot * c_w) : 0.f;
  }
}

// x0[j][i] = local + w_i coef[j][a_i].  A thread per node walks the sets, so
// each access is coalesced across the warp and the node's weight and cluster
// are read once.  (The caller clears the push scratch afterwards with one
// memset: clearing it here, line by line after the read, was several times
// slower than the whole pass.)
__global__ void compose_kernel(long long *push, const float *w, const int32_t *cluster, const float *coef,
                               const int32_t *over, int64_t n, int r, int64_t nsets, float *x0) {
  const float inv_n = 1.0f / (float)n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float wi = w[i];
    const int c = cluster[i];
#pragma unroll 4
    for (int64_t j = 0; j < nsets; ++j) {
      const int64_t q = j * n + i;
      const long long f = __ldcs(&push[q]);
      float v = fix40_to_float(f);
      const int o = over[j];
      if (o == 2) v = inv_n;
      else if (o == 0) v += wi * __ldg(&coef[j * r + c]);
      __stcs(&x0[q], v);
    }
  }
}

// t[j][i] = x*[j][i] - local (in place); the caller clears the push scratch
__global__ void tail_targets(const long long *push, int64_t n, int64_t nsets, float *t) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
#pragma unroll 4
    for (int64_t j = 0; j < nsets; ++j) {
      const int64_t q = j * n + i;
      t[q] -= fix40_to_float(__ldcs(&push[q]));
    }
}

// ymass[j][c] = sum over the members of cluster c of t[j][i] (warp per (j, c), member order)
__global__ void cluster_mass(const float *t, const int32_t *members, const int32_t *off, int r, int64_t n,
                             int64_t nsets, double *ymass) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); q < nsets * r; q += nw) {
    const int64_t j = q / r;
    const int c = (int)(q % r);
    double s = 0.0;
    for (int i = off[c] + lane; i < off[c + 1]; i += 32) s += (double)t[j * n + members[i]];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) ymass[q] = s;
  }
}

// gram += X^T X and rhs += X^T Y over the sets of a chunk (cold sets skipped);
// one thread per output entry, sets in order
__global__ void gram_accumulate(const double *mix, const double *ymass, const int32_t *over, int64_t nsets, int r,
                                double *gram, double *rhs) {
  const int F = 2 * r + 1;
  const int64_t ng = (int64_t)F * F, total = ng + (int64_t)F * r;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    if (q < ng) {
      const int a = (int)(q / F), b = (int)(q % F);
      for (int64_t j = 0; j < nsets; ++j)
        if (over[j] == 0) s += mix[j * F + a] * mix[j * F + b];
      gram[q] += s;
    } else {
      const int64_t q2 = q - ng;
      const int a = (int)(q2 / r), c = (int)(q2 % r);
      for (int64_t j = 0; j < nsets; ++j)
        if (over[j] == 0) s += mix[j * F + a] * ymass[j * r + c];
      rhs[q2] += s;
    }
  }
}

// K = (G + lambda I)^-1 R by Cholesky factorisation, one CTA, FP64
__global__ void __launch_bounds__(1024) ls_solve(const double *gram, const double *rhs, int F, int r, double ridge,
                                                 double *A, float *K) {
  __shared__ double lam;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int64_t q = tid; q < (int64_t)F * F; q += nt) A[q] = gram[q];
  __syncthreads();
  if (tid == 0) {
    double tr = 0.0;
    for (int i = 0; i < F; ++i) tr += A[(int64_t)i * F + i];
    lam = ridge * (tr > 0.0 ? tr / F : 1.0) + 1e-300;
  }
  __syncthreads();
  for (int i = tid; i < F; i += nt) A[(int64_t)i * F + i] += lam;
  __syncthreads();
  for (int k = 0; k < F; ++k) {
    if (tid == 0) A[(int64_t)k * F + k] = sqrt(fmax(A[(int64_t)k * F + k], 1e-300));
    __syncthreads();
    const double dk = A[(int64_t)k * F + k];
    for (int i = k + 1 + tid; i < F; i += nt) A[(int64_t)i * F + k] /= dk;
    __syncthreads();
    const int m = F - k - 1;
    for (int64_t q = tid; q < (int64_t)m * m; q += nt) {
      const int i = k + 1 + (int)(q / m), j = k + 1 + (int)(q % m);
      if (j <= i) A[(int64_t)i * F + j] -= A[(int64_t)i * F + k] * A[(int64_t)j * F + k];
    }
    __syncthreads();
  }
  // L y = R, then L^T K = y, one right-hand column per thread; y (FP64)
  // lives after the factor in A
  double *y = A + (int64_t)F * F;
  for (int c = tid; c < r; c += nt) {
    for (int f = 0; f < F; ++f) {
      double t = rhs[(int64_t)f * r + c];
      for (int g = 0; g < f; ++g) t -= A[(int64_t)f * F + g] * y[(int64_t)g * r + c];
      y[(int64_t)f * r + c] = t / A[(int64_t)f * F + f];
    }
    for (int f = F - 1; f >= 0; --f) {
      double t = y[(int64_t)f * r + c];
      for (int g = f + 1; g < F; ++g) t -= A[(int64_t)g * F + f] * y[(int64_t)g * r + c];
      y[(int64_t)f * r + c] = t / A[(int64_t)f * F + f];
      K[(int64_t)f * r + c] = (float)y[(int64_t)f * r + c];
    }
  }
}

// ---- loss: mean over sets of || tail_pred - tail ||_1 and dL/du
// pass A: residual signs, per-node part of dL/dw, loss partials
__global__ void loss_a(const float *t, const float *w, const int32_t *cluster, const float *coef, int r, int64_t n,
                       int B, int8_t *gsign, float *tpart, double *lpart) {
  __shared__ float cs[kWMaxBatch * kWMaxClusters];
  __shared__ double red[256];
  for (int q = threadIdx.x; q < B * r; q += blockDim.x) cs[q] = coef[q];
  __syncthreads();
  double loss = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = cluster[i];
    const float wi = w[i];
    float t1 = 0.f;
    for (int j = 0; j < B; ++j) {
      const float cf = cs[j * r + c];
      const float e = wi * cf - t[(int64_t)j * n + i];
      const int8_t g = e > 0.f ? 1 : (e < 0.f ? -1 : 0);
      gsign[(int64_t)j * n + i] = g;
      loss += fabs((double)e);
      t1 += (float)g * cf;
    }
    tpart[i] = t1;
  }
  red[threadIdx.x] = loss;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) lpart[blockIdx.x] = red[0];
}

// pass B: csum[j][c] = sum over cluster c of sign * w (warp per (j, c), member order)
__global__ void loss_b(const int8_t *gsign, const float *w, const int32_t *members, const int32_t *off, int r,
                       int64_t n, int B, float *csum) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); q < (int64_t)B * r; q += nw) {
    const int64_t j = q / r;
    const int c = (int)(q % r);
    float s = 0.f;
    for (int i = off[c] + lane; i < off[c + 1]; i += 32) {
      const int32_t v = members[i];
      s += (float)gsign[j * n + v] * w[v];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) csum[q] = s;
  }
}

// pass C: du_i = w_i/B * (tpart_i - sum_j coef[j][a_i] csum[j][a_i] / cw[a_i]);
// no gradient where u sits at its clamp
__global__ void loss_c(const float *tpart, const float *w, const int32_t *cluster, const float *coef, const float *csum,
                       const float *cw, int r, int64_t n, int B, float *du) {
  const float lo = expf(-20.f) * 1.000001f, hi = expf(20.f) * 0.999999f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = cluster[i];
    float s = 0.f;
    for (int j = 0; j < B; ++j) s += coef[j * r + c] * csum[j * r + c];
    const float wi = w[i];
    const float dw = tpart[i] - (cw[c] > 0.f ? s / cw[c] : 0.f);
    du[i] = (wi <= lo || wi >= hi) ? 0.f : dw * wi / (float)B;
  }
}

double wall_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

WarmModel::~WarmModel() {
  void *ptrs[] = {out_rp, out_col, in_rp, in_col, inv_out, inv_in, code, x1, cluster, members, cl_off,
                  params, adam_m, adam_v, w1t, w2t, w2, coupling, h1, a1, h2, g2, gx, w, du, cw, grad, part,
                  push, mix, tmass, r1c, over, coef, d_sptr, d_sidx, t3, t4, targets, gsign, csum, ymass, gram,
                  rhs, chol, lpart, x0};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (tc_err_h) cudaFreeHost(tc_err_h);
}

namespace {

Status col_standardize(WarmModel &w, float *a, int C) {
  cudaStream_t s = w.ctx->stream;
  const int threads = (256 / C) * C;
  const int blocks = blocks_for(w.n * C, threads, 1024);
  double *part = nullptr;
  GOPS_CUDA_TRY(cudaMalloc(&part, sizeof(double) * blocks * 2 * C));
  col_stats<<<blocks, threads, 0, s>>>(a, w.n, C, part);
  std::vector<double> h((size_t)blocks * 2 * C);
  cudaError_t e = cudaMemcpyAsync(h.data(), part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(part);
  GOPS_CUDA_TRY(e);
  std::vector<float> mean(C), isd(C);
  for (int k = 0; k < C; ++k) {
    double su = 0.0, sq = 0.0;
    for (int b = 0; b < blocks; ++b) {
      su += h[(size_t)b * 2 * C + k];
      sq += h[(size_t)b * 2 * C + C + k];
    }
    const double mu = su / (double)w.n;
    const double var = std::max(sq / (double)w.n - mu * mu, 0.0);
    mean[k] = (float)mu;
    isd[k] = var > 1e-30 ? (float)(1.0 / std::sqrt(var)) : 1.0f;
  }
  float *dm = nullptr;
  GOPS_CUDA_TRY(cudaMalloc(&dm, sizeof(float) * 2 * C));
  e = cudaMemcpyAsync(dm, mean.data(), sizeof(float) * C, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dm + C, isd.data(), sizeof(float) * C, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    col_apply<<<blocks_for(w.n * C, 256, 4096), 256, 0, s>>>(a, w.n, C, dm, dm + C);
    e = cudaStreamSynchronize(s);
  }
  cudaFree(dm);
  GOPS_CUDA_TRY(e);
  return Status::ok();
}

Status kmeans(WarmModel &w, const float *y) {
  cudaStream_t s = w.ctx->stream;
  const int64_t n = w.n;
  const int r = w.r;
  float *cent = nullptr, *d2 = nullptr;
  double *cs = nullptr;
  long long *sums = nullptr;
  int *counts = nullptr;
  const int64_t nch = (n + kChunk - 1) / kChunk;
  struct Guard {
    std::vector<void *> p;
    ~Guard() {
      for (void *q : p) cudaFree(q);
    }
  } guard;
  GOPS_CUDA_TRY(cudaMalloc(&cent, sizeof(float) * r * kWY));
  guard.p.push_back(cent);
  GOPS_CUDA_TRY(cudaMalloc(&d2, sizeof(float) * n));
  guard.p.push_back(d2);
  GOPS_CUDA_TRY(cudaMalloc(&cs, sizeof(double) * nch));
  guard.p.push_back(cs);
  GOPS_CUDA_TRY(cudaMalloc(&sums, sizeof(long long) * r * kWY));
  guard.p.push_back(sums);
  GOPS_CUDA_TRY(cudaMalloc(&counts, sizeof(int) * r));
  guard.p.push_back(counts);
  int32_t *assign = nullptr;
  GOPS_CUDA_TRY(cudaMalloc(&assign, sizeof(int32_t) * n));
  guard.p.push_back(assign);
  std::vector<double> hcs(nch);
  std::vector<float> hd(kChunk);
  const int gb = blocks_for(n, 256, w.ctx->num_sms * 8);
  const size_t smem = sizeof(float) * r * kWY + sizeof(long long) * r * kWY + sizeof(int) * r;
  GOPS_CUDA_TRY(cudaFuncSetAttribute(km_assign, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int ab = std::max(1, w.ctx->num_sms);
  // kKmeansRestarts seeded runs; the one with the smallest within-cluster sum
  // of squares is kept (ties: the earliest)
  double best_inertia = INFINITY;
  for (int rs = 0; rs < kKmeansRestarts; ++rs) {
    // k-means++ seeding
    uint64_t ctr = mix64(w.cfg.seed ^ 0xC1A55EEDull ^ (rs ? mix64((uint64_t)rs) : 0ull));
    auto uniform = [&]() { return (double)(mix64(ctr++) >> 11) * (1.0 / 9007199254740992.0); };
    int64_t idx = (int64_t)(uniform() * (double)n);
    if (idx >= n) idx = n - 1;
    for (int t = 0; t < r; ++t) {
      GOPS_CUDA_TRY(cudaMemcpyAsync(cent + (int64_t)t * kWY, y + idx * kWY, sizeof(float) * kWY,
                                    cudaMemcpyDeviceToDevice, s));
      if (t == r - 1) break;
      kmpp_dist<<<gb, 256, 0, s>>>(y, n, cent + (int64_t)t * kWY, t == 0, d2);
      chunk_sums<<<(unsigned)nch, 256, 0, s>>>(d2, n, cs);
      GOPS_CUDA_TRY(cudaMemcpyAsync(hcs.data(), cs, sizeof(double) * nch, cudaMemcpyDeviceToHost, s));
      GOPS_CUDA_TRY(cudaStreamSynchronize(s));
      double total = 0.0;
      for (int64_t c = 0; c < nch; ++c) total += hcs[c];
      const double u = uniform();
      if (!(total > 0.0)) {
        idx = std::min<int64_t>(n - 1, (int64_t)(u * (double)n));
        continue;
      }
      double target = u * total, run = 0.0;
      int64_t ch = 0;
      while (ch < nch - 1 && run + hcs[ch] <= target) run += hcs[ch++];
      const int64_t base = ch * kChunk, len = std::min<int64_t>(kChunk, n - base);
      GOPS_CUDA_TRY(cudaMemcpyAsync(hd.data(), d2 + base, sizeof(float) * len, cudaMemcpyDeviceToHost, s));
      GOPS_CUDA_TRY(cudaStreamSynchronize(s));
      // the same per-thread order as chunk_sums is not needed here: pick the
      // first node whose running sum passes the target, else the last positive one
      idx = -1;
      int64_t last_pos = -1;
      for (int64_t q = 0; q < len; ++q) {
        if (hd[q] > 0.f) last_pos = base + q;
        run += (double)hd[q];
        if (run > target && hd[q] > 0.f) {
          idx = base + q;
          break;
        }
      }
      if (idx < 0) idx = last_pos >= 0 ? last_pos : base;
    }
    // Lloyd iterations; the last pass only assigns and records each node's
    // squared distance to its centroid
    for (int it = 0; it <= w.cfg.kmeans_iters; ++it) {
      const bool upd = it < w.cfg.kmeans_iters;
      if (upd) {
        GOPS_CUDA_TRY(cudaMemsetAsync(sums, 0, sizeof(long long) * r * kWY, s));
        GOPS_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(int) * r, s));
      }
      km_assign<<<ab, 256, smem, s>>>(y, n, cent, r, assign, upd ? sums : nullptr, counts, upd ? nullptr : d2);
      GOPS_CUDA_TRY(cudaGetLastError());
      if (upd) km_update<<<(r * kWY + 255) / 256, 256, 0, s>>>(cent, r, sums, counts);
    }
    chunk_sums<<<(unsigned)nch, 256, 0, s>>>(d2, n, cs);
    GOPS_CUDA_TRY(cudaMemcpyAsync(hcs.data(), cs, sizeof(double) * nch, cudaMemcpyDeviceToHost, s));
    GOPS_CUDA_TRY(cudaStreamSynchronize(s));
    double inertia = 0.0;
    for (int64_t c = 0; c < nch; ++c) inertia += hcs[c];
    if (inertia < best_inertia || rs == 0) {
      best_inertia = inertia;
      GOPS_CUDA_TRY(cudaMemcpyAsync(w.cluster, assign, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
    }
  }
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  return Status::ok();
}

Status build_members(WarmModel &w) {
  cudaStream_t s = w.ctx->stream;
  const int64_t n = w.n;
  uint32_t *k1 = nullptr, *v1 = nullptr, *k2 = nullptr, *v2 = nullptr;
  struct Guard {
    std::vector<void *> p;
    ~Guard() {
      for (void *q : p) cudaFree(q);
    }
  } guard;
  GOPS_CUDA_TRY(cudaMalloc(&k1, sizeof(uint32_t) * n));
  guard.p.push_back(k1);
  GOPS_CUDA_TRY(cudaMalloc(&v1, sizeof(uint32_t) * n));
  guard.p.push_back(v1);
  GOPS_CUDA_TRY(cudaMalloc(&k2, sizeof(uint32_t) * n));
  guard.p.push_back(k2);
  GOPS_CUDA_TRY(cudaMalloc(&v2, sizeof(uint32_t) * n));
  guard.p.push_back(v2);
  GOPS_CUDA_TRY(cudaMemcpyAsync(k1, w.cluster, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s));
  iota_u32<<<blocks_for(n, 256, 4096), 256, 0, s>>>(v1, n);
  bool alt = false;
  GOPS_TRY(radix_sort_pairs_u32(k1, v1, k2, v2, n, 8, &alt, s));
  const uint32_t *ks = alt ? k2 : k1;
  const uint32_t *vs = alt ? v2 : v1;
  GOPS_CUDA_TRY(cudaMemcpyAsync(w.members, vs, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s));
  int64_t *off64 = nullptr;
  GOPS_CUDA_TRY(cudaMalloc(&off64, sizeof(int64_t) * (w.r + 1)));
  guard.p.push_back(off64);
  offsets_from_sorted<<<blocks_for(n + 1, 256, 4096), 256, 0, s>>>(ks, n, w.r, off64);
  std::vector<int64_t> h(w.r + 1);
  GOPS_CUDA_TRY(cudaMemcpyAsync(h.data(), off64, sizeof(int64_t) * (w.r + 1), cudaMemcpyDeviceToHost, s));
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  std::vector<int32_t> h32(h.begin(), h.end());
  GOPS_CUDA_TRY(cudaMemcpyAsync(w.cl_off, h32.data(), sizeof(int32_t) * (w.r + 1), cudaMemcpyHostToDevice, s));
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  return Status::ok();
}

// the tables t3 and t4: sparse runs of the 1- and 2-step cluster
// distributions h and h2 (count, scan, fill per level), then t3 from h2 and
// t4 from t3; the runs are freed afterwards
Status build_tables(WarmModel &w) {
  cudaStream_t s = w.ctx->stream;
  const int64_t n = w.n;
  const size_t smem = sizeof(long long) * 8 * w.r;
  const int grid = blocks_for(n, 8, w.ctx->num_sms * 32);
  int64_t *rp[2] = {nullptr, nullptr};
  int32_t *cl[2] = {nullptr, nullptr};
  float *wt[2] = {nullptr, nullptr};
  struct Guard {
    int64_t **rp;
    int32_t **cl;
    float **wt;
    ~Guard() {
      for (int l = 0; l < 2; ++l) {
        cudaFree(rp[l]);
        cudaFree(cl[l]);
        cudaFree(wt[l]);
      }
    }
  } guard{rp, cl, wt};
  for (int level = 1; level <= 2; ++level) {
    const int L = level - 1;
    GOPS_CUDA_TRY(cudaMalloc(&rp[L], sizeof(int64_t) * (n + 1)));
    GOPS_CUDA_TRY(cudaMemsetAsync(rp[L] + n, 0, sizeof(int64_t), s));
    for (int fill = 0; fill < 2; ++fill) {
      if (fill) {
        GOPS_TRY(exclusive_scan_i64(rp[L], rp[L], n + 1, s));
        int64_t total = 0;
        GOPS_CUDA_TRY(cudaMemcpyAsync(&total, rp[L] + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        GOPS_CUDA_TRY(cudaStreamSynchronize(s));
        GOPS_CUDA_TRY(cudaMalloc(&cl[L], sizeof(int32_t) * std::max<int64_t>(total, 1)));
        GOPS_CUDA_TRY(cudaMalloc(&wt[L], sizeof(float) * std::max<int64_t>(total, 1)));
      }
      if (level == 1)
        runs_kernel<1><<<grid, 256, smem, s>>>(w.out_rp, w.out_col, w.inv_out, w.cluster, nullptr, nullptr, nullptr,
                                               n, w.r, rp[0], cl[0], wt[0], fill);
      else
        runs_kernel<2><<<grid, 256, smem, s>>>(w.out_rp, w.out_col, w.inv_out, w.cluster, rp[0], cl[0], wt[0], n,
                                               w.r, rp[1], cl[1], wt[1], fill);
      GOPS_CUDA_TRY(cudaGetLastError());
    }
  }
  GOPS_CUDA_TRY(cudaMalloc(&w.t3, sizeof(float) * n * w.r));
  GOPS_CUDA_TRY(cudaMalloc(&w.t4, sizeof(float) * n * w.r));
  table_from_runs<<<grid, 256, smem, s>>>(w.out_rp, w.out_col, w.inv_out, rp[1], cl[1], wt[1], n, w.r, w.t3);
  table_next<<<grid, 256, 0, s>>>(w.out_rp, w.out_col, w.inv_out, w.t3, n, w.r, w.t4);
  GOPS_CUDA_TRY(cudaGetLastError());
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  return Status::ok();
}

Status ensure_sets(WarmModel &w, int64_t sets) {
  if (sets <= w.set_cap) return Status::ok();
  cudaFree(w.mix); cudaFree(w.tmass); cudaFree(w.r1c); cudaFree(w.over); cudaFree(w.coef); cudaFree(w.ymass);
  w.mix = nullptr; w.tmass = nullptr; w.r1c = nullptr; w.over = nullptr; w.coef = nullptr; w.ymass = nullptr;
  w.set_cap = 0;
  const int F = 2 * w.r + 1;
  GOPS_CUDA_TRY(cudaMalloc(&w.mix, sizeof(double) * sets * F));
  GOPS_CUDA_TRY(cudaMalloc(&w.tmass, sizeof(double) * sets));
  GOPS_CUDA_TRY(cudaMalloc(&w.r1c, sizeof(double) * sets));
  GOPS_CUDA_TRY(cudaMalloc(&w.over, sizeof(int32_t) * sets));
  GOPS_CUDA_TRY(cudaMalloc(&w.coef, sizeof(float) * sets * w.r));
  GOPS_CUDA_TRY(cudaMalloc(&w.ymass, sizeof(double) * sets * w.r));
  w.set_cap = sets;
  return Status::ok();
}

Status ensure_push(WarmModel &w, int64_t sets) {
  GOPS_TRY(ensure_sets(w, sets));
  if (sets <= w.push_cap) return Status::ok();
  cudaFree(w.push);
  w.push = nullptr;
  w.push_cap = 0;
  GOPS_CUDA_TRY(cudaMalloc(&w.push, sizeof(long long) * sets * w.n));
  GOPS_CUDA_TRY(cudaMemsetAsync(w.push, 0, sizeof(long long) * sets * w.n, w.ctx->stream));
  w.push_cap = sets;
  return Status::ok();
}

// seed sets [s0, s0 + cnt) to the device, offsets rebased to 0
Status upload_sets(WarmModel &w, const int64_t *sptr, const int32_t *sidx, int64_t s0, int64_t cnt) {
  cudaStream_t s = w.ctx->stream;
  const int64_t b = sptr[s0], e = sptr[s0 + cnt];
  if (cnt + 1 > w.sptr_cap) {
    cudaFree(w.d_sptr);
    w.d_sptr = nullptr;
    w.sptr_cap = 0;
    GOPS_CUDA_TRY(cudaMalloc(&w.d_sptr, sizeof(int64_t) * (cnt + 1)));
    w.sptr_cap = cnt + 1;
  }
  if (e - b > w.sidx_cap || !w.d_sidx) {
    cudaFree(w.d_sidx);
    w.d_sidx = nullptr;
    w.sidx_cap = 0;
    GOPS_CUDA_TRY(cudaMalloc(&w.d_sidx, sizeof(int32_t) * std::max<int64_t>(e - b, 1)));
    w.sidx_cap = std::max<int64_t>(e - b, 1);
  }
  std::vector<int64_t> rb(cnt + 1);
  for (int64_t q = 0; q <= cnt; ++q) rb[q] = sptr[s0 + q] - b;
  GOPS_CUDA_TRY(cudaMemcpyAsync(w.d_sptr, rb.data(), sizeof(int64_t) * (cnt + 1), cudaMemcpyHostToDevice, s));
  if (e > b) GOPS_CUDA_TRY(cudaMemcpyAsync(w.d_sidx, sidx + b, sizeof(int32_t) * (e - b), cudaMemcpyHostToDevice, s));
  w.ctx->stats.h2d_bytes += sizeof(int64_t) * (cnt + 1) + sizeof(int32_t) * (e - b);
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));  // rb lives on this stack frame
  return Status::ok();
}

Status run_push(WarmModel &w, double damping, int64_t cnt) {
  PushArgs a{w.out_rp, w.out_col, w.inv_out, w.t3, w.t4, w.cluster, w.d_sptr, w.d_sidx, w.n, w.r, (float)damping,
             w.cfg.push_budget, w.push, w.mix, w.tmass, w.r1c, w.over};
  static bool attr = false;
  if (!attr) {
    GOPS_CUDA_TRY(cudaFuncSetAttribute(push_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(PushSmem)));
    attr = true;
  }
  push_kernel<<<(unsigned)cnt, kPushThreads, sizeof(PushSmem), w.ctx->stream>>>(a);
  GOPS_CUDA_TRY(cudaGetLastError());
  return Status::ok();
}

Status run_coef(WarmModel &w, int64_t s0, int64_t cnt) {
  const int F = 2 * w.r + 1;
  coef_kernel<<<(unsigned)cnt, 256, 0, w.ctx->stream>>>(w.mix + s0 * F, w.coupling, w.cw, w.tmass + s0, w.over + s0,
                                                       w.r, w.coef + s0 * w.r);
  GOPS_CUDA_TRY(cudaGetLastError());
  return Status::ok();
}

Status fit_coupling(WarmModel &w) {
  const int F = 2 * w.r + 1;
  ls_solve<<<1, 1024, 0, w.ctx->stream>>>(w.gram, w.rhs, F, w.r, (double)w.cfg.ridge, w.chol, w.coupling);
  GOPS_CUDA_TRY(cudaGetLastError());
  w.coupling_set = true;
  return Status::ok();
}

Status ensure_train(WarmModel &w, int64_t chunk) {
  GOPS_TRY(ensure_push(w, chunk));
  const int F = 2 * w.r + 1;
  if (chunk > w.targets_cap) {
    cudaFree(w.targets);
    w.targets = nullptr;
    w.targets_cap = 0;
    GOPS_CUDA_TRY(cudaMalloc(&w.targets, sizeof(float) * chunk * w.n));
    w.targets_cap = chunk;
  }
  if (!w.gsign) GOPS_CUDA_TRY(cudaMalloc(&w.gsign, sizeof(int8_t) * kWMaxBatch * w.n));
  if (!w.csum) GOPS_CUDA_TRY(cudaMalloc(&w.csum, sizeof(float) * kWMaxBatch * w.r));
  if (!w.gram || !w.rhs || !w.chol) {  // all three, or none after a failed attempt
    cudaFree(w.gram); cudaFree(w.rhs); cudaFree(w.chol);
    w.gram = nullptr; w.rhs = nullptr; w.chol = nullptr;
    GOPS_CUDA_TRY(cudaMalloc(&w.gram, sizeof(double) * F * F));
    GOPS_CUDA_TRY(cudaMalloc(&w.rhs, sizeof(double) * F * w.r));
    GOPS_CUDA_TRY(cudaMalloc(&w.chol, sizeof(double) * ((int64_t)F * F + (int64_t)F * w.r)));
    GOPS_CUDA_TRY(cudaMemsetAsync(w.gram, 0, sizeof(double) * F * F, w.ctx->stream));
    GOPS_CUDA_TRY(cudaMemsetAsync(w.rhs, 0, sizeof(double) * F * w.r, w.ctx->stream));
  }
  if (!w.lpart) GOPS_CUDA_TRY(cudaMalloc(&w.lpart, sizeof(double) * 4096));
  return Status::ok();
}

// loss and du for sets [s0, s0 + B) of the current chunk (targets hold tails)
Status loss_grad(WarmModel &w, const float *tails, int64_t s0, int B, double *loss) {
  cudaStream_t s = w.ctx->stream;
  const int lb = blocks_for(w.n, 256, std::min(4096, w.ctx->num_sms * 8));
  loss_a<<<lb, 256, 0, s>>>(tails, w.w, w.cluster, w.coef + s0 * w.r, w.r, w.n, B, w.gsign, w.du, w.lpart);
  loss_b<<<blocks_for((int64_t)B * w.r, 8, 4096), 256, 0, s>>>(w.gsign, w.w, w.members, w.cl_off, w.r, w.n, B, w.csum);
  loss_c<<<blocks_for(w.n, 256, 4096), 256, 0, s>>>(w.du, w.w, w.cluster, w.coef + s0 * w.r, w.csum, w.cw, w.r, w.n, B,
                                                   w.du);
  GOPS_CUDA_TRY(cudaGetLastError());
  if (loss) {
    std::vector<double> h(lb);
    GOPS_CUDA_TRY(cudaMemcpyAsync(h.data(), w.lpart, sizeof(double) * lb, cudaMemcpyDeviceToHost, s));
    GOPS_CUDA_TRY(cudaStreamSynchronize(s));
    double t = 0.0;
    for (double v : h) t += v;
    *loss = t / (double)B;
  }
  return Status::ok();
}

}  // namespace

// ---------------------------------------------------------------------------
// drivers
// ---------------------------------------------------------------------------
Status warm_create(Ctx *ctx, const Graph *g, const int64_t *row_ptr, const int32_t *col, const gops_warm_config *cfg,
                   WarmModel &w) {
  w.ctx = ctx;
  w.device = ctx->device;
  w.graph = g;
  w.cfg = *cfg;
  w.n = g->n;
  w.m = g->m;
  w.r = cfg->clusters;
  const int64_t n = w.n, m = w.m;
  if (n < 1) return Status{GOPS_ERR_INVALID, "warm start: empty graph"};
  if (w.r < 1 || w.r > kWMaxClusters) return Status{GOPS_ERR_INVALID, "warm start: clusters must be in 1..256"};
  if (w.r > n) w.r = (int)n;
  if (cfg->minibatch < 1 || cfg->minibatch > kWMaxBatch)
    return Status{GOPS_ERR_INVALID, "warm start: minibatch must be in 1..32"};
  if (cfg->chunk < cfg->minibatch) return Status{GOPS_ERR_INVALID, "warm start: chunk must be >= minibatch"};
  if (cfg->code_steps < 0 || cfg->kmeans_iters < 0 || cfg->epochs < 0 || !(cfg->lr > 0.f) || !(cfg->ridge >= 0.f) ||
      cfg->push_budget < 0)
    return Status{GOPS_ERR_INVALID, "warm start: invalid configuration"};
  if (row_ptr[n] != m) return Status{GOPS_ERR_INVALID, "warm start: row_ptr does not match the graph"};
  cudaStream_t s = ctx->stream;
  GOPS_CUDA_TRY(cudaMalloc(&w.out_rp, sizeof(int64_t) * (n + 1)));
  GOPS_CUDA_TRY(cudaMalloc(&w.out_col, sizeof(int32_t) * std::max<int64_t>(m, 1)));
  GOPS_CUDA_TRY(cudaMalloc(&w.in_rp, sizeof(int64_t) * (n + 1)));
  GOPS_CUDA_TRY(cudaMalloc(&w.in_col, sizeof(int32_t) * std::max<int64_t>(m, 1)));
  GOPS_CUDA_TRY(cudaMalloc(&w.inv_out, sizeof(float) * n));
  GOPS_CUDA_TRY(cudaMalloc(&w.inv_in, sizeof(float) * n));
  GOPS_CUDA_TRY(cudaMalloc(&w.code, sizeof(float) * n * kWCode));
  GOPS_CUDA_TRY(cudaMalloc(&w.x1, sizeof(bf16) * n * kWIn));
  GOPS_CUDA_TRY(cudaMalloc(&w.cluster, sizeof(int32_t) * n));
  GOPS_CUDA_TRY(cudaMalloc(&w.members, sizeof(int32_t) * n));
  GOPS_CUDA_TRY(cudaMalloc(&w.cl_off, sizeof(int32_t) * (w.r + 1)));
  GOPS_CUDA_TRY(cudaMalloc(&w.coupling, sizeof(float) * (2 * w.r + 1) * w.r));
  GOPS_CUDA_TRY(cudaMemsetAsync(w.coupling, 0, sizeof(float) * (2 * w.r + 1) * w.r, s));
  GOPS_CUDA_TRY(cudaMemcpyAsync(w.out_rp, row_ptr, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, s));
  if (m) GOPS_CUDA_TRY(cudaMemcpyAsync(w.out_col, col, sizeof(int32_t) * m, cudaMemcpyHostToDevice, s));
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  // in-edge CSR in original order: stable sort of the edges by destination
  {
    uint32_t *k1 = nullptr, *v1 = nullptr, *k2 = nullptr, *v2 = nullptr;
    const int64_t mm = std::max<int64_t>(m, 1);
    GOPS_CUDA_TRY(cudaMalloc(&k1, sizeof(uint32_t) * mm));
    GOPS_CUDA_TRY(cudaMalloc(&v1, sizeof(uint32_t) * mm));
    GOPS_CUDA_TRY(cudaMalloc(&k2, sizeof(uint32_t) * mm));
    GOPS_CUDA_TRY(cudaMalloc(&v2, sizeof(uint32_t) * mm));
    copy_keys<<<blocks_for(m, 256, 8192), 256, 0, s>>>(w.out_col, m, k1);
    expand_src<<<blocks_for(n, 8, 8192), 256, 0, s>>>(w.out_rp, n, v1);
    bool alt = false;
    int bits = 1;
    while (bits < 32 && (int64_t(1) << bits) < n) ++bits;
    Status st = radix_sort_pairs_u32(k1, v1, k2, v2, m, bits, &alt, s);
    if (st.code == GOPS_OK) {
      const uint32_t *ks = alt ? k2 : k1, *vs = alt ? v2 : v1;
      cudaMemcpyAsync(w.in_col, vs, sizeof(int32_t) * m, cudaMemcpyDeviceToDevice, s);
      offsets_from_sorted<<<blocks_for(m + 1, 256, 8192), 256, 0, s>>>(ks, m, n, w.in_rp);
      cudaStreamSynchronize(s);
    }
    cudaFree(k1); cudaFree(v1); cudaFree(k2); cudaFree(v2);
    GOPS_TRY(st);
    GOPS_CUDA_TRY(cudaGetLastError());
  }
  degree_terms<<<blocks_for(n, 256, 8192), 256, 0, s>>>(w.out_rp, w.in_rp, n, w.inv_out, w.inv_in);
  GOPS_CUDA_TRY(cudaGetLastError());
  // random-projection code: Gaussian columns diffused over the graph
  float *tmp = nullptr;
  GOPS_CUDA_TRY(cudaMalloc(&tmp, sizeof(float) * n * kWY));
  struct Tmp {
    float *p;
    ~Tmp() { cudaFree(p); }
  } tguard{tmp};
  code_init<<<blocks_for(n * kWCode, 256, 8192), 256, 0, s>>>(n * kWCode, mix64(cfg->seed), w.code);
  for (int t = 0; t < cfg->code_steps; ++t) {
    code_step<<<blocks_for(n, 16, 8192), 256, 0, s>>>(w.in_rp, w.in_col, w.inv_in, w.out_rp, w.out_col, w.inv_out,
                                                      w.code, n, tmp);
    GOPS_CUDA_TRY(cudaMemcpyAsync(w.code, tmp, sizeof(float) * n * kWCode, cudaMemcpyDeviceToDevice, s));
    GOPS_TRY(col_standardize(w, w.code, kWCode));
  }
  // node features and the layer-1 input
  {
    float *x = nullptr, *ax = nullptr;
    GOPS_CUDA_TRY(cudaMalloc(&x, sizeof(float) * n * kWFeat));
    GOPS_CUDA_TRY(cudaMalloc(&ax, sizeof(float) * n * kWFeat));
    base_features<<<blocks_for(n, 256, 8192), 256, 0, s>>>(w.out_rp, w.in_rp, w.code, n, x);
    Status st = col_standardize(w, x, kWFeat);
    if (st.code == GOPS_OK) {
      agg_small<<<blocks_for(n, 8, 8192), 256, 0, s>>>(w.in_rp, w.in_col, w.inv_in, x, kWFeat, n, ax, kWFeat);
      pack_x1<<<blocks_for(n * kWIn, 256, 8192), 256, 0, s>>>(x, ax, n, w.x1);
      // clustering space [code, mean_in code]
      agg_small<<<blocks_for(n, 8, 8192), 256, 0, s>>>(w.in_rp, w.in_col, w.inv_in, w.code, kWCode, n, ax, kWCode);
      pack_y<<<blocks_for(n * kWY, 256, 8192), 256, 0, s>>>(w.code, ax, n, tmp);
      cudaStreamSynchronize(s);
    }
    cudaFree(x);
    cudaFree(ax);
    GOPS_TRY(st);
    GOPS_CUDA_TRY(cudaGetLastError());
  }
  GOPS_TRY(kmeans(w, tmp));
  GOPS_TRY(build_members(w));
  GOPS_TRY(build_tables(w));
  GOPS_TRY(nn_alloc(w));
  GOPS_TRY(nn_init_params(w));
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  return Status::ok();
}

Status warm_train(WarmModel &w, const gops_config *cfg, int64_t nsets, const int64_t *seed_ptr,
                  const int32_t *seed_idx, gops_warm_stats *stats) {
  Ctx *ctx = w.ctx;
  cudaStream_t s = ctx->stream;
  const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(w.cfg.chunk, nsets));
  GOPS_TRY(ensure_train(w, chunk));
  gops_warm_stats st{};
  double t_targets = 0.0, t_fit = 0.0;
  bool first_loss = true;
  const int F = 2 * w.r + 1;
  std::vector<int32_t> over_h(chunk);
  for (int ep = 0; ep < std::max(1, w.cfg.epochs); ++ep) {
    for (int64_t c0 = 0; c0 < nsets; c0 += chunk) {
      const int64_t cnt = std::min(chunk, nsets - c0);
      // targets: the sets' PPR vectors from the batched solver
      const double ta = wall_ms();
      GOPS_TRY(ppr_batch(ctx, const_cast<Graph *>(w.graph), cfg, cnt, seed_ptr + c0, seed_idx, nullptr, false,
                         w.targets, true, nullptr, nullptr, nullptr));
      GOPS_CUDA_TRY(cudaStreamSynchronize(s));
      const double tb = wall_ms();
      t_targets += tb - ta;
      st.sets += cnt;
      // exact part, tails, cluster masses, normal equations
      GOPS_TRY(upload_sets(w, seed_ptr, seed_idx, c0, cnt));
      GOPS_TRY(run_push(w, cfg->damping, cnt));
      tail_targets<<<blocks_for(w.n, 256, w.ctx->num_sms * 8), 256, 0, s>>>(w.push, w.n, cnt, w.targets);
      GOPS_CUDA_TRY(cudaMemsetAsync(w.push, 0, sizeof(long long) * cnt * w.n, s));
      if (ep == 0) {
        cluster_mass<<<blocks_for(cnt * w.r, 8, 8192), 256, 0, s>>>(w.targets, w.members, w.cl_off, w.r, w.n, cnt,
                                                                     w.ymass);
        gram_accumulate<<<blocks_for((int64_t)F * F + (int64_t)F * w.r, 256, 4096), 256, 0, s>>>(
            w.mix, w.ymass, w.over, cnt, w.r, w.gram, w.rhs);
        GOPS_CUDA_TRY(cudaGetLastError());
        w.gram_sets += cnt;
        GOPS_TRY(fit_coupling(w));
      }
      GOPS_CUDA_TRY(cudaMemcpyAsync(over_h.data(), w.over, sizeof(int32_t) * cnt, cudaMemcpyDeviceToHost, s));
      GOPS_CUDA_TRY(cudaStreamSynchronize(s));
      // Adam steps over minibatches of the chunk's warm-startable sets
      std::vector<int64_t> ok;
      for (int64_t j = 0; j < cnt; ++j)
        if (over_h[j] == 0) ok.push_back(j);
      for (size_t b0 = 0; b0 + w.cfg.minibatch <= ok.size(); b0 += w.cfg.minibatch) {
        // the minibatch's sets must be contiguous in the chunk: take runs
        const int64_t j0 = ok[b0];
        if (ok[b0 + w.cfg.minibatch - 1] != j0 + w.cfg.minibatch - 1) continue;
        GOPS_TRY(nn_forward(w));
        GOPS_TRY(run_coef(w, j0, w.cfg.minibatch));
        double loss = 0.0;
        const bool want = first_loss || b0 + 2 * w.cfg.minibatch > ok.size();
        GOPS_TRY(loss_grad(w, w.targets + j0 * w.n, j0, w.cfg.minibatch, want ? &loss : nullptr));
        if (want) {
          if (first_loss) st.loss_first = loss;
          st.loss_last = loss;
          first_loss = false;
        }
        GOPS_TRY(nn_backward(w));
        GOPS_TRY(nn_adam(w, w.cfg.lr));
        ++st.steps;
      }
      GOPS_CUDA_TRY(cudaStreamSynchronize(s));
      GOPS_TRY(nn_check(w));
      t_fit += wall_ms() - tb;
    }
  }
  GOPS_TRY(nn_forward(w));
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  GOPS_TRY(nn_check(w));
  st.target_ms = t_targets;
  st.fit_ms = t_fit;
  if (stats) *stats = st;
  return Status::ok();
}

Status warm_predict(WarmModel &w, double damping, int64_t nsets, const int64_t *seed_ptr, const int32_t *seed_idx,
                    float *x0, double *r1_cold) {
  cudaStream_t s = w.ctx->stream;
  if (!w.weights_fresh) {
    GOPS_TRY(nn_forward(w));
    GOPS_CUDA_TRY(cudaStreamSynchronize(s));
    GOPS_TRY(nn_check(w));
  }
  const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(nsets, std::max<int64_t>(w.cfg.chunk, 1)));
  GOPS_TRY(ensure_push(w, chunk));
  for (int64_t c0 = 0; c0 < nsets; c0 += chunk) {
    const int64_t cnt = std::min(chunk, nsets - c0);
    GOPS_TRY(upload_sets(w, seed_ptr, seed_idx, c0, cnt));
    GOPS_TRY(run_push(w, damping, cnt));
    GOPS_TRY(run_coef(w, 0, cnt));
    compose_kernel<<<blocks_for(w.n, 256, w.ctx->num_sms * 8), 256, 0, s>>>(w.push, w.w, w.cluster, w.coef, w.over,
                                                                             w.n, w.r, cnt, x0 + c0 * w.n);
    GOPS_CUDA_TRY(cudaGetLastError());
    GOPS_CUDA_TRY(cudaMemsetAsync(w.push, 0, sizeof(long long) * cnt * w.n, s));
    if (r1_cold) {
      GOPS_CUDA_TRY(cudaMemcpyAsync(r1_cold + c0, w.r1c, sizeof(double) * cnt, cudaMemcpyDeviceToHost, s));
      GOPS_CUDA_TRY(cudaStreamSynchronize(s));
    }
  }
  return Status::ok();
}

// batched PPR from caller warm starts (device, set-major) judged by their
// first residual: a set whose step-1 residual is not below r1_max is
// retired and solved again from its personalization vector
Status judged_batch(Ctx *ctx, Graph *g, const gops_config *cfg, int64_t nsets, const int64_t *seed_ptr,
                    const int32_t *seed_idx, const float *x0_dev, const double *r1_max, float *scores,
                    bool scores_on_device, gops_run *runs, int32_t *rejected) {
  cudaStream_t s = ctx->stream;
  const int64_t n = g->n;
  std::vector<int32_t> rej(nsets, 0);
  std::vector<gops_run> rr(nsets);
  GOPS_TRY(ppr_batch(ctx, g, cfg, nsets, seed_ptr, seed_idx, x0_dev, true, scores, scores_on_device, rr.data(),
                     r1_max, rej.data()));
  gops_stats agg = ctx->stats;
  std::vector<int64_t> redo;
  for (int64_t q = 0; q < nsets; ++q)
    if (rej[q]) redo.push_back(q);
  if (!redo.empty()) {
    const int64_t nr = (int64_t)redo.size();
    std::vector<int64_t> sp(nr + 1, 0);
    std::vector<int32_t> si;
    for (int64_t q = 0; q < nr; ++q) {
      for (int64_t k = seed_ptr[redo[q]]; k < seed_ptr[redo[q] + 1]; ++k) si.push_back(seed_idx[k]);
      sp[q + 1] = (int64_t)si.size();
    }
    std::vector<gops_run> r2(nr);
    float *tmp = nullptr;
    if (scores) GOPS_CUDA_TRY(cudaMalloc(&tmp, sizeof(float) * nr * n));
    Status st2 = ppr_batch(ctx, g, cfg, nr, sp.data(), si.empty() ? nullptr : si.data(), nullptr, false, tmp, true,
                           r2.data(), nullptr, nullptr);
    if (st2.code == GOPS_OK && scores) {
      for (int64_t q = 0; q < nr && st2.code == GOPS_OK; ++q) {
        const cudaError_t e = cudaMemcpyAsync(scores + redo[q] * n, tmp + q * n, sizeof(float) * n,
                                              scores_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) st2 = Status{GOPS_ERR_CUDA, cudaGetErrorString(e)};
      }
      if (st2.code == GOPS_OK) {
        const cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st2 = Status{GOPS_ERR_CUDA, cudaGetErrorString(e)};
      }
    }
    if (tmp) cudaFree(tmp);
    GOPS_TRY(st2);
    for (int64_t q = 0; q < nr; ++q) rr[redo[q]] = r2[q];
    agg.solve_ms += ctx->stats.solve_ms;
    agg.kernel_launches += ctx->stats.kernel_launches;
    agg.iterations += ctx->stats.iterations;
    agg.h2d_bytes += ctx->stats.h2d_bytes;
    agg.d2h_bytes += ctx->stats.d2h_bytes;
  }
  ctx->stats = agg;
  if (runs)
    for (int64_t q = 0; q < nsets; ++q) runs[q] = rr[q];
  if (rejected)
    for (int64_t q = 0; q < nsets; ++q) rejected[q] = rej[q];
  return Status::ok();
}

Status warm_batch(WarmModel &w, const gops_config *cfg, int64_t nsets, const int64_t *seed_ptr,
                  const int32_t *seed_idx, float *scores, bool scores_on_device, gops_run *runs, int32_t *rejected) {
  Ctx *ctx = w.ctx;
  cudaStream_t s = ctx->stream;
  if (nsets <= 0) return Status::ok();
  if (nsets > w.x0_cap) {
    cudaFree(w.x0);
    w.x0 = nullptr;
    w.x0_cap = 0;
    GOPS_CUDA_TRY(cudaMalloc(&w.x0, sizeof(float) * nsets * w.n));
    w.x0_cap = nsets;
  }
  std::vector<double> r1(nsets);
  const uint64_t h2d0 = ctx->stats.h2d_bytes;
  GOPS_CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
  GOPS_TRY(warm_predict(w, cfg->damping, nsets, seed_ptr, seed_idx, w.x0, r1.data()));
  GOPS_CUDA_TRY(cudaEventRecord(ctx->ev[2], s));
  GOPS_CUDA_TRY(cudaEventSynchronize(ctx->ev[2]));
  float t_pred = 0.f;
  cudaEventElapsedTime(&t_pred, ctx->ev[1], ctx->ev[2]);
  const uint64_t h2d_pred = ctx->stats.h2d_bytes - h2d0;
  GOPS_TRY(judged_batch(ctx, const_cast<Graph *>(w.graph), cfg, nsets, seed_ptr, seed_idx, w.x0, r1.data(), scores,
                        scores_on_device, runs, rejected));
  ctx->stats.solve_ms += t_pred;
  ctx->stats.h2d_bytes += h2d_pred;
  return Status::ok();
}

Status warm_loss_grad(WarmModel &w, double damping, int64_t nsets, const int64_t *seed_ptr, const int32_t *seed_idx,
                      const float *targets_x, double *loss, float *grad) {
  cudaStream_t s = w.ctx->stream;
  if (nsets < 1 || nsets > kWMaxBatch) return Status{GOPS_ERR_INVALID, "loss_grad: nsets must be in 1..32"};
  GOPS_TRY(ensure_train(w, nsets));
  GOPS_CUDA_TRY(cudaMemcpyAsync(w.targets, targets_x, sizeof(float) * nsets * w.n, cudaMemcpyHostToDevice, s));
  GOPS_TRY(upload_sets(w, seed_ptr, seed_idx, 0, nsets));
  GOPS_TRY(run_push(w, damping, nsets));
  tail_targets<<<blocks_for(w.n, 256, w.ctx->num_sms * 8), 256, 0, s>>>(w.push, w.n, nsets, w.targets);
  GOPS_CUDA_TRY(cudaMemsetAsync(w.push, 0, sizeof(long long) * nsets * w.n, s));
  GOPS_TRY(nn_forward(w));
  GOPS_TRY(run_coef(w, 0, nsets));
  GOPS_TRY(loss_grad(w, w.targets, 0, (int)nsets, loss));
  GOPS_TRY(nn_backward(w));
  GOPS_CUDA_TRY(cudaMemcpyAsync(grad, w.grad, sizeof(float) * kPCount, cudaMemcpyDeviceToHost, s));
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  return nn_check(w);
}

Status warm_push_one(WarmModel &w, double damping, const int32_t *seeds, int64_t nseeds, double *local, double *mix,
                     double *tail_mass, double *r1_cold) {
  cudaStream_t s = w.ctx->stream;
  GOPS_TRY(ensure_push(w, 1));
  const int64_t sp[2] = {0, nseeds};
  GOPS_TRY(upload_sets(w, sp, seeds, 0, 1));
  GOPS_TRY(run_push(w, damping, 1));
  std::vector<long long> h(w.n);
  int32_t ov = 0;
  GOPS_CUDA_TRY(cudaMemcpyAsync(h.data(), w.push, sizeof(long long) * w.n, cudaMemcpyDeviceToHost, s));
  GOPS_CUDA_TRY(cudaMemcpyAsync(&ov, w.over, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  if (mix) GOPS_CUDA_TRY(cudaMemcpyAsync(mix, w.mix, sizeof(double) * (2 * w.r + 1), cudaMemcpyDeviceToHost, s));
  if (tail_mass) GOPS_CUDA_TRY(cudaMemcpyAsync(tail_mass, w.tmass, sizeof(double), cudaMemcpyDeviceToHost, s));
  if (r1_cold) GOPS_CUDA_TRY(cudaMemcpyAsync(r1_cold, w.r1c, sizeof(double), cudaMemcpyDeviceToHost, s));
  GOPS_CUDA_TRY(cudaMemsetAsync(w.push, 0, sizeof(long long) * w.n, s));
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  if (local)
    for (int64_t i = 0; i < w.n; ++i) local[i] = (double)h[i] / kWFix;
  if (ov) return Status{GOPS_ERR_INVALID, "push: the set exceeds the push budget"};
  return Status::ok();
}

}  // namespace gops

// ---------------------------------------------------------------------------
// extern "C" entry points (include/gops.h)
// ---------------------------------------------------------------------------
using namespace gops;

namespace {

inline float bf16_bits_to_float(uint16_t b) {
  const uint32_t u = (uint32_t)b << 16;
  float f;
  std::memcpy(&f, &u, sizeof f);
  return f;
}

int warm_guard(gops_ctx *ctx, gops_warm *w) {
  if (!ctx || !w) return GOPS_ERR_INVALID;
  if (w->impl.ctx != &ctx->impl) return ctx->impl.set(Status{GOPS_ERR_INVALID, "model belongs to another context"});
  cudaSetDevice(ctx->impl.device);
  return GOPS_OK;
}

Status check_sets(int64_t n, int64_t nsets, const int64_t *seed_ptr, const int32_t *seed_idx) {
  if (nsets < 0) return Status{GOPS_ERR_INVALID, "nsets must be >= 0"};
  if (nsets == 0) return Status::ok();
  if (!seed_ptr) return Status{GOPS_ERR_INVALID, "seed_ptr is NULL"};
  for (int64_t s = 0; s < nsets; ++s)
    if (seed_ptr[s + 1] < seed_ptr[s]) return Status{GOPS_ERR_INVALID, "seed_ptr must be non-decreasing"};
  if (seed_ptr[nsets] > seed_ptr[0] && !seed_idx) return Status{GOPS_ERR_INVALID, "seed_idx is NULL"};
  for (int64_t k = seed_ptr[0]; k < seed_ptr[nsets]; ++k)
    if (seed_idx[k] < 0 || seed_idx[k] >= n) return Status{GOPS_ERR_INVALID, "seed index out of range"};
  return Status::ok();
}

Status check_damping(double d) {
  if (!std::isfinite(d) || d < 0.0 || d > 1.0) return Status{GOPS_ERR_INVALID, "damping must be in [0,1]"};
  return Status::ok();
}

}  // namespace

extern "C" {

void gops_warm_config_default(gops_warm_config *cfg) {
  if (!cfg) return;
  cfg->clusters = 128;
  cfg->code_steps = 10;
  cfg->kmeans_iters = 20;
  cfg->minibatch = 32;
  cfg->chunk = 512;
  cfg->epochs = 1;
  cfg->lr = 3e-3f;
  cfg->ridge = 1e-9f;
  cfg->seed = 0x9E3779B97F4A7C15ull;
  cfg->push_budget = int64_t(1) << 24;
}

int gops_warm_create(gops_ctx *ctx, const gops_graph *g, const int64_t *row_ptr, const int32_t *col,
                     const gops_warm_config *wcfg, gops_warm **out) {
  if (!ctx) return GOPS_ERR_INVALID;
  Ctx &c = ctx->impl;
  if (!g || !row_ptr || !out) return c.set(Status{GOPS_ERR_INVALID, "null argument"});
  if (g->impl.ctx != &c) return c.set(Status{GOPS_ERR_INVALID, "graph belongs to another context"});
  *out = nullptr;
  gops_warm_config cfg;
  gops_warm_config_default(&cfg);
  if (wcfg) cfg = *wcfg;
  if (g->impl.m > 0 && !col) return c.set(Status{GOPS_ERR_INVALID, "col is NULL"});
  for (int64_t u = 0; u < g->impl.n; ++u)
    if (row_ptr[u + 1] < row_ptr[u]) return c.set(Status{GOPS_ERR_INVALID, "row_ptr must be non-decreasing"});
  for (int64_t e = 0; e < row_ptr[g->impl.n]; ++e)
    if (col[e] < 0 || col[e] >= g->impl.n) return c.set(Status{GOPS_ERR_INVALID, "neighbor index out of range"});
  cudaSetDevice(c.device);
  gops_warm *w = new (std::nothrow) gops_warm();
  if (!w) return c.set(Status{GOPS_ERR_OOM, "host allocation failed"});
  const Status st = warm_create(&c, &g->impl, row_ptr, col, &cfg, w->impl);
  if (st.code != GOPS_OK) {
    delete w;
    return c.set(st);
  }
  *out = w;
  return GOPS_OK;
}

void gops_warm_destroy(gops_warm *w) {
  if (!w) return;
  // the context may already be gone: use the device recorded at creation
  // (cudaFree waits for the device's pending work before it frees)
  cudaSetDevice(w->impl.device);
  delete w;
}

int gops_warm_train(gops_ctx *ctx, gops_warm *w, const gops_config *cfg, int64_t nsets, const int64_t *seed_ptr,
                    const int32_t *seed_idx, gops_warm_stats *stats) {
  if (int rc = warm_guard(ctx, w)) return rc;
  Ctx &c = ctx->impl;
  if (!cfg) return c.set(Status{GOPS_ERR_INVALID, "null argument"});
  if (int rc = gops_config_validate(cfg, nullptr, 0)) return c.set(Status{rc, "invalid configuration"});
  Status st = check_sets(w->impl.n, nsets, seed_ptr, seed_idx);
  if (st.code == GOPS_OK) st = warm_train(w->impl, cfg, nsets, seed_ptr, seed_idx, stats);
  return c.set(st);
}

int gops_warm_predict(gops_ctx *ctx, gops_warm *w, double damping, int64_t nsets, const int64_t *seed_ptr,
                      const int32_t *seed_idx, float *x0_device, double *r1_cold) {
  if (int rc = warm_guard(ctx, w)) return rc;
  Ctx &c = ctx->impl;
  if (nsets > 0 && !x0_device) return c.set(Status{GOPS_ERR_INVALID, "x0_device is NULL"});
  Status st = check_damping(damping);
  if (st.code == GOPS_OK) st = check_sets(w->impl.n, nsets, seed_ptr, seed_idx);
  if (st.code == GOPS_OK && nsets > 0)
    st = warm_predict(w->impl, damping, nsets, seed_ptr, seed_idx, x0_device, r1_cold);
  return c.set(st);
}

static int learned_common(gops_ctx *ctx, const gops_graph *g, gops_warm *w, const gops_config *cfg, int64_t nsets,
                          const int64_t *seed_ptr, const int32_t *seed_idx, float *scores, bool on_device,
                          gops_run *runs, int32_t *rejected) {
  if (int rc = warm_guard(ctx, w)) return rc;
  Ctx &c = ctx->impl;
  if (!g || !cfg) return c.set(Status{GOPS_ERR_INVALID, "null argument"});
  if (&g->impl != w->impl.graph) return c.set(Status{GOPS_ERR_INVALID, "model was built for another graph"});
  if (int rc = gops_config_validate(cfg, nullptr, 0)) return c.set(Status{rc, "invalid configuration"});
  Status st = check_sets(w->impl.n, nsets, seed_ptr, seed_idx);
  if (st.code == GOPS_OK)
    st = warm_batch(w->impl, cfg, nsets, seed_ptr, seed_idx, scores, on_device, runs, rejected);
  return c.set(st);
}

int gops_ppr_batch_learned(gops_ctx *ctx, const gops_graph *g, gops_warm *w, const gops_config *cfg, int64_t nsets,
                           const int64_t *seed_ptr, const int32_t *seed_idx, float *scores, gops_run *runs,
                           int32_t *rejected) {
  return learned_common(ctx, g, w, cfg, nsets, seed_ptr, seed_idx, scores, false, runs, rejected);
}

int gops_ppr_batch_learned_device(gops_ctx *ctx, const gops_graph *g, gops_warm *w, const gops_config *cfg,
                                  int64_t nsets, const int64_t *seed_ptr, const int32_t *seed_idx,
                                  float *scores_device, gops_run *runs, int32_t *rejected) {
  return learned_common(ctx, g, w, cfg, nsets, seed_ptr, seed_idx, scores_device, true, runs, rejected);
}

int gops_ppr_batch_judged_device(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg, int64_t nsets,
                                 const int64_t *seed_ptr, const int32_t *seed_idx, const float *x0_device,
                                 const double *r1_max, float *scores_device, gops_run *runs, int32_t *rejected) {
  if (!ctx) return GOPS_ERR_INVALID;
  Ctx &c = ctx->impl;
  if (!g || !cfg || (nsets > 0 && !x0_device)) return c.set(Status{GOPS_ERR_INVALID, "null argument"});
  if (g->impl.ctx != &c) return c.set(Status{GOPS_ERR_INVALID, "graph belongs to another context"});
  if (int rc = gops_config_validate(cfg, nullptr, 0)) return c.set(Status{rc, "invalid configuration"});
  cudaSetDevice(c.device);
  Status st = check_sets(g->impl.n, nsets, seed_ptr, seed_idx);
  if (st.code == GOPS_OK && nsets > 0)
    st = judged_batch(&c, const_cast<Graph *>(&g->impl), cfg, nsets, seed_ptr, seed_idx, x0_device, r1_max,
                      scores_device, true, runs, rejected);
  return c.set(st);
}

int64_t gops_warm_count(const gops_warm *w, int what) {
  if (!w) return -1;
  const WarmModel &m = w->impl;
  switch (what) {
    case GOPS_WARM_PARAMS: return kPCount;
    case GOPS_WARM_COUPLING: return (int64_t)(2 * m.r + 1) * m.r;
    case GOPS_WARM_CLUSTERS: return m.n;
    case GOPS_WARM_FEATURES: return m.n * kWIn;
    case GOPS_WARM_CODE: return m.n * kWCode;
    case GOPS_WARM_WEIGHT: return m.n;
    default: return -1;
  }
}

int gops_warm_get(gops_ctx *ctx, gops_warm *w, int what, void *host, int64_t count) {
  if (int rc = warm_guard(ctx, w)) return rc;
  Ctx &c = ctx->impl;
  WarmModel &m = w->impl;
  const int64_t need = gops_warm_count(w, what);
  if (need < 0 || !host || count != need) return c.set(Status{GOPS_ERR_INVALID, "bad field or count"});
  cudaStream_t s = c.stream;
  Status st;
  auto copy = [&](const void *src, size_t bytes) -> Status {
    GOPS_CUDA_TRY(cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, s));
    GOPS_CUDA_TRY(cudaStreamSynchronize(s));
    return Status::ok();
  };
  switch (what) {
    case GOPS_WARM_PARAMS: st = copy(m.params, sizeof(float) * need); break;
    case GOPS_WARM_COUPLING: st = copy(m.coupling, sizeof(float) * need); break;
    case GOPS_WARM_CLUSTERS: st = copy(m.cluster, sizeof(int32_t) * need); break;
    case GOPS_WARM_CODE: st = copy(m.code, sizeof(float) * need); break;
    case GOPS_WARM_WEIGHT:
      if (!m.weights_fresh) st = nn_forward(m);
      if (st.code == GOPS_OK) st = copy(m.w, sizeof(float) * need);
      break;
    case GOPS_WARM_FEATURES: {
      std::vector<uint16_t> b(need);
      const cudaError_t e1 = cudaMemcpyAsync(b.data(), m.x1, sizeof(uint16_t) * need, cudaMemcpyDeviceToHost, s);
      const cudaError_t e2 = e1 == cudaSuccess ? cudaStreamSynchronize(s) : e1;
      if (e2 != cudaSuccess) {
        st = Status{GOPS_ERR_CUDA, cudaGetErrorString(e2)};
        break;
      }
      float *o = static_cast<float *>(host);
      for (int64_t i = 0; i < need; ++i) o[i] = bf16_bits_to_float(b[i]);
      break;
    }
  }
  return c.set(st);
}

int gops_warm_set(gops_ctx *ctx, gops_warm *w, int what, const void *host, int64_t count) {
  if (int rc = warm_guard(ctx, w)) return rc;
  Ctx &c = ctx->impl;
  WarmModel &m = w->impl;
  const int64_t need = gops_warm_count(w, what);
  if ((what != GOPS_WARM_PARAMS && what != GOPS_WARM_COUPLING) || !host || count != need)
    return c.set(Status{GOPS_ERR_INVALID, "bad field or count"});
  const float *f = static_cast<const float *>(host);
  for (int64_t i = 0; i < need; ++i)
    if (!std::isfinite(f[i])) return c.set(Status{GOPS_ERR_INVALID, "values must be finite"});
  cudaStream_t s = c.stream;
  auto run = [&]() -> Status {
    if (what == GOPS_WARM_PARAMS) {
      GOPS_CUDA_TRY(cudaMemcpyAsync(m.params, host, sizeof(float) * need, cudaMemcpyHostToDevice, s));
      GOPS_CUDA_TRY(cudaMemsetAsync(m.adam_m, 0, sizeof(float) * kPCount, s));
      GOPS_CUDA_TRY(cudaMemsetAsync(m.adam_v, 0, sizeof(float) * kPCount, s));
      m.adam_t = 0;
      GOPS_TRY(nn_refresh_bf16(m));
    } else {
      GOPS_CUDA_TRY(cudaMemcpyAsync(m.coupling, host, sizeof(float) * need, cudaMemcpyHostToDevice, s));
      m.coupling_set = true;
    }
    GOPS_CUDA_TRY(cudaStreamSynchronize(s));
    return Status::ok();
  };
  return c.set(run());
}

int gops_warm_loss_grad(gops_ctx *ctx, gops_warm *w, double damping, int64_t nsets, const int64_t *seed_ptr,
                        const int32_t *seed_idx, const float *targets_x, double *loss, float *grad) {
  if (int rc = warm_guard(ctx, w)) return rc;
  Ctx &c = ctx->impl;
  if (!targets_x || !grad) return c.set(Status{GOPS_ERR_INVALID, "null argument"});
  Status st = check_damping(damping);
  if (st.code == GOPS_OK) st = check_sets(w->impl.n, nsets, seed_ptr, seed_idx);
  if (st.code == GOPS_OK) st = warm_loss_grad(w->impl, damping, nsets, seed_ptr, seed_idx, targets_x, loss, grad);
  return c.set(st);
}

int gops_warm_push(gops_ctx *ctx, gops_warm *w, double damping, const int32_t *seeds, int64_t nseeds, double *local,
                   double *mix, double *tail_mass, double *r1_cold) {
  if (int rc = warm_guard(ctx, w)) return rc;
  Ctx &c = ctx->impl;
  const int64_t sp[2] = {0, nseeds};
  Status st = check_damping(damping);
  if (st.code == GOPS_OK) st = check_sets(w->impl.n, 1, sp, seeds);
  if (st.code == GOPS_OK) st = warm_push_one(w->impl, damping, seeds, nseeds, local, mix, tail_mass, r1_cold);
  return c.set(st);
}

}  // extern "C"
