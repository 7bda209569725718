// top_k and normalize (src/topk.rs:17-61) on device-resident scores: the
// k largest finite positive scores of each row, by score descending.  The
// reference keeps, at the boundary, the entries met first (a later equal score
// does not displace a kept one) and leaves the order of equal scores
// unspecified; here equal scores are ordered by index, which selects the same
// set and makes the output deterministic.
//
// One CTA per segment of a row, the segment held in registers (16,384 FP32
// or 8,192 FP64 entries: 32 or 16 per thread).  Finite positive IEEE values
// order like their bit patterns, so the selection runs on those keys.  A
// lower bound T on the k-th largest key comes from the per-thread maxima
// (every warp sorts its 32 maxima with shuffles; with m = ceil(take / 16), at
// least m threads of each of the 16 warps hold a key >= their warp's m-th
// largest maximum, so T = the least of those leaves at least take keys >= T).
// The keys >= T (a few hundred for typical score vectors) go to shared memory
// and a bitonic sort by (key desc, index asc) leaves the answer in the first
// `take` slots.  When more than kCap keys pass T (heavy ties, or k above the
// bound's reach), a bisection on the key bits over the registers finds the
// k-th largest key exactly (32 or 64 block-wide counts), and every key above
// it plus the lowest-index keys equal to it are sorted the same way.
// Rows longer than one segment run in stages: every segment's top k, then
// the top k of the row's candidates, until one segment holds them.  The
// result is the same: every key of the row's top k is in its segment's top k
// (fewer than k keys of the row exceed the k-th largest, and each segment
// keeps its lowest-index equal keys up to k), and the candidates come in
// segment order, each segment's sorted by index among equal keys, so the
// lowest candidate position among equal keys is the lowest row index.
#include <cstdint>

#include "objects.cuh"

namespace gops {
namespace {

constexpr int kTThreads = 512;
constexpr int kTWarps = kTThreads / 32;
constexpr int kMaxK = 1024;
constexpr int kCap = 2048;                 // candidates sorted in shared memory
constexpr int64_t kRowsPerLaunch = 16384;  // rows per launch (grid size = rows x segments)

template <class V>
struct KeyOf;
template <>
struct KeyOf<float> {
  using K = uint32_t;
  static constexpr int kBits = 32;
  static constexpr int kE = 32;  // keys per thread
  __device__ static K key(float v) { return (isfinite(v) && v > 0.f) ? __float_as_uint(v) : 0u; }
};
template <>
struct KeyOf<double> {
  using K = unsigned long long;
  static constexpr int kBits = 64;
  static constexpr int kE = 16;
  __device__ static K key(double v) {
    return (isfinite(v) && v > 0.0) ? (K)__double_as_longlong(v) : 0ull;
  }
};
template <class V>
constexpr int64_t seg_cap() {
  return (int64_t)kTThreads * KeyOf<V>::kE;
}

// sum of one int per thread over the block (every thread gets it); sred
// holds kTWarps ints and is free again on return
__device__ __forceinline__ int block_sum(int v, int *sred) {
  v = (int)__reduce_add_sync(0xffffffffu, (unsigned)v);
  if ((threadIdx.x & 31) == 0) sred[threadIdx.x >> 5] = v;
  __syncthreads();
  int t = 0;
#pragma unroll
  for (int w = 0; w < kTWarps; ++w) t += sred[w];
  __syncthreads();
  return t;
}

// Block (r, b) = blockIdx.x = r * nseg + b takes entries [b * C, min(n_row,
// (b + 1) * C)) of row r (rows row_stride apart; C = seg_cap<V>()) and writes
// k entries at blockIdx.x * k: the top `take` by (key desc, index asc), their
// row indices (through idx_map when given), then padding (value 0: not a
// key; index -1); count_out[blockIdx.x] = take.
template <class V>
__global__ void __launch_bounds__(kTThreads, 2) topk_rows(const V *__restrict__ x, int64_t row_stride, int64_t n_row,
                                                       int nseg, int k, const int64_t *__restrict__ idx_map,
                                                       int64_t *__restrict__ idx_out, V *__restrict__ val_out,
                                                       int64_t *__restrict__ count_out) {
  using KO = KeyOf<V>;
  using K = typename KO::K;
  constexpr int E = KO::kE;
  constexpr int64_t C = seg_cap<V>();
  __shared__ K ck[kCap];
  __shared__ int cidx[kCap];
  __shared__ int sred[kTWarps];
  __shared__ K s_tw[kTWarps];
  __shared__ int s_cnt, s_eqbase;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int64_t r = blockIdx.x / nseg, seg = blockIdx.x % nseg;
  const int64_t off = r * row_stride + seg * C;
  const V *row = x + off;
  const int n = (int)min(C, n_row - seg * C);
  const int64_t o = (int64_t)blockIdx.x * k;
  // entry j * kTThreads + tid of the segment, 0 beyond it
  K key[E];
#pragma unroll
  for (int j = 0; j < E; ++j) {
    const int i = j * kTThreads + tid;
    key[j] = i < n ? KO::key(row[i]) : (K)0;
  }
  K mx = 0;
  int cnt = 0;
#pragma unroll
  for (int j = 0; j < E; ++j) {
    cnt += key[j] != 0;
    mx = key[j] > mx ? key[j] : mx;
  }
  const int valid = block_sum(cnt, sred);
  const int take = valid < k ? valid : k;
  if (take == 0) {
    for (int i = tid; i < k; i += kTThreads) {
      idx_out[o + i] = -1;
      val_out[o + i] = (V)0;
    }
    if (tid == 0) count_out[blockIdx.x] = 0;
    return;
  }
  // lower bound T from the thread maxima (descending bitonic sort per warp)
  const int m = (take + kTWarps - 1) / kTWarps;
  if (m <= 32) {
#pragma unroll
    for (int size = 2; size <= 32; size <<= 1)
#pragma unroll
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        const K other = __shfl_xor_sync(0xffffffffu, mx, stride);
        const bool keep_max = ((lane & size) == 0) == ((lane & stride) == 0);
        mx = keep_max ? (mx > other ? mx : other) : (mx < other ? mx : other);
      }
    if (lane == m - 1) s_tw[wid] = mx;
  }
  if (tid == 0) s_cnt = 0;
  __syncthreads();
  K lo = 1;
  if (m <= 32) {
    K t = s_tw[0];
#pragma unroll
    for (int w = 1; w < kTWarps; ++w) t = s_tw[w] < t ? s_tw[w] : t;
    lo = t > 0 ? t : 1;
  }
  int c = 0;
#pragma unroll
  for (int j = 0; j < E; ++j) c += key[j] >= lo;
  c = block_sum(c, sred);
  int nc;
  if (c <= kCap) {
#pragma unroll
    for (int j = 0; j < E; ++j) {
      const bool f = key[j] >= lo;
      const unsigned bal = __ballot_sync(0xffffffffu, f);
      if (bal) {
        const int leader = __ffs(bal) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(&s_cnt, __popc(bal));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (f) {
          const int pos = base + __popc(bal & ((1u << lane) - 1u));
          ck[pos] = key[j];
          cidx[pos] = j * kTThreads + tid;
        }
      }
    }
    nc = c;
  } else {
    // the take-th largest key exactly, by bisection on the key bits: keep a
    // bit when at least `take` keys are >= the prefix with it set
    K thr = 0;
    for (int bit = KO::kBits - 1; bit >= 0; --bit) {
      const K cand = thr | ((K)1 << bit);
      int ge = 0;
#pragma unroll
      for (int j = 0; j < E; ++j) ge += key[j] >= cand;
      if (block_sum(ge, sred) >= take) thr = cand;
    }
    int gt = 0;
#pragma unroll
    for (int j = 0; j < E; ++j) gt += key[j] > thr;
    const int need_eq = take - block_sum(gt, sred);  // keys equal to thr to take (>= 1)
    if (tid == 0) s_eqbase = 0;
    // every key above thr (take - need_eq of them), in any order
#pragma unroll
    for (int j = 0; j < E; ++j) {
      const bool f = key[j] > thr;
      const unsigned bal = __ballot_sync(0xffffffffu, f);
      if (bal) {
        const int leader = __ffs(bal) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(&s_cnt, __popc(bal));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (f) {
          const int pos = base + __popc(bal & ((1u << lane) - 1u));
          ck[pos] = key[j];
          cidx[pos] = j * kTThreads + tid;
        }
      }
    }
    // the need_eq lowest-index keys equal to thr, after them
#pragma unroll
    for (int j = 0; j < E; ++j) {
      const bool eq = key[j] == thr;
      const unsigned bal = __ballot_sync(0xffffffffu, eq);
      if (lane == 0) sred[wid] = __popc(bal);
      __syncthreads();
      int before = s_eqbase;
      for (int w = 0; w < wid; ++w) before += sred[w];
      before += __popc(bal & ((1u << lane) - 1u));
      if (eq && before < need_eq) {
        const int pos = take - need_eq + before;
        ck[pos] = key[j];
        cidx[pos] = j * kTThreads + tid;
      }
      __syncthreads();
      if (tid == 0) {
        int t = 0;
        for (int w = 0; w < kTWarps; ++w) t += sred[w];
        s_eqbase += t;
      }
      __syncthreads();
    }
    nc = take;
  }
  __syncthreads();
  // bitonic sort of the nc candidates by (key desc, index asc), padded to a power of two
  int p2 = 1;
  while (p2 < nc) p2 <<= 1;
  for (int i = nc + tid; i < p2; i += kTThreads) {
    ck[i] = 0;
    cidx[i] = INT32_MAX;
  }
  __syncthreads();
  for (int size = 2; size <= p2; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = tid; i < p2; i += kTThreads) {
        const int j = i ^ stride;
        if (j > i) {
          const bool up = (i & size) == 0;  // this pair's half sorts "first before second"
          // "a before b": larger key, or equal key and smaller index
          const bool a_first = ck[i] > ck[j] || (ck[i] == ck[j] && cidx[i] < cidx[j]);
          if (a_first != up) {
            const K tk = ck[i];
            ck[i] = ck[j];
            ck[j] = tk;
            const int ti = cidx[i];
            cidx[i] = cidx[j];
            cidx[j] = ti;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int i = tid; i < k; i += kTThreads) {
    if (i < take) {
      idx_out[o + i] = idx_map ? idx_map[off + cidx[i]] : seg * C + cidx[i];
      val_out[o + i] = row[cidx[i]];
    } else {
      idx_out[o + i] = -1;
      val_out[o + i] = (V)0;
    }
  }
  if (tid == 0) count_out[blockIdx.x] = take;
}

// normalize (src/topk.rs:53-61): divide by the sum when the sum > 0.  The
// sum in a fixed order: per block of the grid (strided, then a tree), then
// the block sums by one block.
constexpr int kSumBlocks = 1024;
__global__ void sum_f64_part(const double *x, int64_t n, double *part) {
  __shared__ double sh[256];
  double t = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    t += x[i];
  sh[threadIdx.x] = t;
  __syncthreads();
  for (int q = blockDim.x / 2; q > 0; q >>= 1) {
    if ((int)threadIdx.x < q) sh[threadIdx.x] += sh[threadIdx.x + q];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void sum_f64(const double *x, int64_t n, double *out) {
  __shared__ double sh[1024];
  double t = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) t += x[i];
  sh[threadIdx.x] = t;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

__global__ void div_f64(double *x, int64_t n, const double *sum) {
  const double s = *sum;
  if (!(s > 0.0)) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] /= s;
}

template <class V>
Status topk_impl(Ctx *ctx, const V *x, int64_t rows, int64_t n, int64_t k, int64_t *idx, V *val, int64_t *counts) {
  if (rows < 0 || n < 0 || k < 0) return Status{GOPS_ERR_INVALID, "negative size"};
  if (k > kMaxK) return Status{GOPS_ERR_INVALID, "k must be <= 1024"};
  if (rows == 0) return Status::ok();
  if (k == 0 || n == 0) {  // src/topk.rs:18-20
    for (int64_t r = 0; r < rows; ++r) counts[r] = 0;
    return Status::ok();
  }
  cudaStream_t s = ctx->stream;
  int64_t *d_idx = nullptr, *d_cnt = nullptr, *c_idx = nullptr, *c_cnt = nullptr;
  V *d_val = nullptr, *c_val = nullptr;
  Status st;
  auto fail = [&](cudaError_t e) {
    return Status{e == cudaErrorMemoryAllocation ? GOPS_ERR_OOM : GOPS_ERR_CUDA, cudaGetErrorString(e)};
  };
  constexpr int64_t C = seg_cap<V>();
  // stages: segments of C entries -> k candidates each, until one segment per row
  const int64_t nseg1 = ceil_div<int64_t>(n, C);
  const int64_t cand = nseg1 > 1 ? nseg1 * k : 0;  // candidates per row after the first stage
  cudaError_t e = dev_malloc_async((void **)&d_idx, sizeof(int64_t) * rows * k, s);
  if (e == cudaSuccess) e = dev_malloc_async((void **)&d_val, sizeof(V) * rows * k, s);
  if (e == cudaSuccess) e = dev_malloc_async((void **)&d_cnt, sizeof(int64_t) * rows, s);
  if (cand) {  // two candidate buffers, used in turn
    if (e == cudaSuccess) e = dev_malloc_async((void **)&c_idx, sizeof(int64_t) * rows * cand * 2, s);
    if (e == cudaSuccess) e = dev_malloc_async((void **)&c_val, sizeof(V) * rows * cand * 2, s);
    if (e == cudaSuccess) e = dev_malloc_async((void **)&c_cnt, sizeof(int64_t) * rows * nseg1, s);
  }
  for (int64_t r0 = 0; r0 < rows && e == cudaSuccess; r0 += kRowsPerLaunch) {
    const int64_t nr = rows - r0 < kRowsPerLaunch ? rows - r0 : kRowsPerLaunch;
    const V *src = x + r0 * n;
    const int64_t *map = nullptr;
    int64_t len = n;
    for (int buf = 0; e == cudaSuccess; buf ^= 1) {
      const int64_t nseg = ceil_div<int64_t>(len, C);
      if (nseg == 1) {
        topk_rows<V><<<(unsigned)nr, kTThreads, 0, s>>>(src, len, len, 1, (int)k, map, d_idx + r0 * k,
                                                         d_val + r0 * k, d_cnt + r0);
        e = cudaGetLastError();
        break;
      }
      int64_t *oi = c_idx + (int64_t)buf * rows * cand + r0 * nseg * k;
      V *ov = c_val + (int64_t)buf * rows * cand + r0 * nseg * k;
      topk_rows<V><<<(unsigned)(nr * nseg), kTThreads, 0, s>>>(src, len, len, (int)nseg, (int)k, map, oi, ov,
                                                                c_cnt + r0 * nseg);
      e = cudaGetLastError();
      src = ov;
      map = oi;
      len = nseg * k;
    }
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(idx, d_idx, sizeof(int64_t) * rows * k, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(val, d_val, sizeof(V) * rows * k, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(counts, d_cnt, sizeof(int64_t) * rows, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) st = fail(e);
  free_async(d_idx, s);
  free_async(d_val, s);
  free_async(d_cnt, s);
  free_async(c_idx, s);
  free_async(c_val, s);
  free_async(c_cnt, s);
  cudaStreamSynchronize(s);
  return st;
}

}  // namespace
}  // namespace gops

using namespace gops;

extern "C" {

int gops_top_k_f64_device(gops_ctx *ctx, const double *scores_device, int64_t n, int64_t k, int64_t *idx,
                          double *val, int64_t *count) {
  if (!ctx) return GOPS_ERR_INVALID;
  Ctx &c = ctx->impl;
  if ((n > 0 && !scores_device) || !idx || !val || !count) return c.set(Status{GOPS_ERR_INVALID, "null argument"});
  cudaSetDevice(c.device);
  return c.set(topk_impl<double>(&c, scores_device, 1, n, k, idx, val, count));
}

int gops_top_k_f32_rows_device(gops_ctx *ctx, const float *block_device, int64_t rows, int64_t n, int64_t k,
                               int64_t *idx, float *val, int64_t *counts) {
  if (!ctx) return GOPS_ERR_INVALID;
  Ctx &c = ctx->impl;
  if ((rows > 0 && n > 0 && !block_device) || !idx || !val || !counts)
    return c.set(Status{GOPS_ERR_INVALID, "null argument"});
  cudaSetDevice(c.device);
  return c.set(topk_impl<float>(&c, block_device, rows, n, k, idx, val, counts));
}

int gops_normalize_f64_device(gops_ctx *ctx, double *scores_device, int64_t n) {
  if (!ctx) return GOPS_ERR_INVALID;
  Ctx &c = ctx->impl;
  if (n < 0 || (n > 0 && !scores_device)) return c.set(Status{GOPS_ERR_INVALID, "null argument"});
  if (n == 0) return GOPS_OK;
  cudaSetDevice(c.device);
  double *d_sum = nullptr;
  const int nb = blocks_for(n, 256, kSumBlocks);
  cudaError_t e = dev_malloc_async((void **)&d_sum, sizeof(double) * (nb + 1), c.stream);
  if (e == cudaSuccess) {
    sum_f64_part<<<nb, 256, 0, c.stream>>>(scores_device, n, d_sum + 1);
    sum_f64<<<1, 1024, 0, c.stream>>>(d_sum + 1, nb, d_sum);
    div_f64<<<blocks_for(n, 256, 4096), 256, 0, c.stream>>>(scores_device, n, d_sum);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  free_async(d_sum, c.stream);
  cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return c.set(Status{GOPS_ERR_CUDA, cudaGetErrorString(e)});
  return GOPS_OK;
}

}  // extern "C"
