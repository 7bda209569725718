// top_k and normalize (src/topk.rs:17-61) on device-resident scores: the
// k largest finite positive scores of each row, by score descending.  The
// reference keeps, at the boundary, the entries met first (a later equal score
// does not displace a kept one) and leaves the order of equal scores
// unspecified; here equal scores are ordered by index, which selects the same
// set and makes the output deterministic.
//
// One CTA per segment of a row: an MSB-first radix select on the value's bit
// pattern (finite positive IEEE values order like their bits) finds the k-th
// largest key in 4 (FP32) or 8 (FP64) passes of 8 bits over the segment; a
// collection pass takes every key above it and the lowest-index keys equal
// to it; a bitonic sort in shared memory orders the at most k survivors.
// Rows longer than two segments run in two stages, so that a row spreads
// over many SMs: every segment's top k (stage 1), then the top k of the
// row's candidates (stage 2).  The result is the same: every key of the
// row's top k is in its segment's top k (fewer than k keys of the row exceed
// the k-th largest, and each segment keeps its lowest-index equal keys up to
// k), and the candidates come in segment order, each segment's sorted by
// index among equal keys, so the lowest candidate position among equal keys
// is the lowest row index.
#include <cstdint>

#include "objects.cuh"

namespace gops {
namespace {

constexpr int kTThreads = 512;
constexpr int kMaxK = 1024;
constexpr int64_t kSegLen = 32768;        // entries per segment of a long row
constexpr int64_t kRowsPerLaunch = 16384;  // rows per launch (grid size = rows x segments)

template <class V>
struct KeyOf;
template <>
struct KeyOf<float> {
  using K = uint32_t;
  static constexpr int kBits = 32;
  __device__ static K key(float v) { return (isfinite(v) && v > 0.f) ? __float_as_uint(v) : 0u; }
};
template <>
struct KeyOf<double> {
  using K = unsigned long long;
  static constexpr int kBits = 64;
  __device__ static K key(double v) {
    return (isfinite(v) && v > 0.0) ? (K)__double_as_longlong(v) : 0ull;
  }
};

// Block (r, b) = blockIdx.x = r * nseg + b takes entries [b * seg_len,
// min(n, (b + 1) * seg_len)) of row r (rows row_stride apart) and writes k
// entries at blockIdx.x * k: the top `take` by (key desc, index asc), their
// row indices (through idx_map when given), then padding (value 0: not a
// key; index -1); count_out[blockIdx.x] = take.
template <class V>
__global__ void __launch_bounds__(kTThreads) topk_rows(const V *__restrict__ x, int64_t row_stride, int64_t seg_len,
                                                       int64_t n_row, int nseg, int k,
                                                       const int64_t *__restrict__ idx_map,
                                                       int64_t *__restrict__ idx_out, V *__restrict__ val_out,
                                                       int64_t *__restrict__ count_out) {
  using KO = KeyOf<V>;
  using K = typename KO::K;
  __shared__ unsigned hist[256];
  __shared__ K s_prefix;
  __shared__ int s_need;     // how many keys >= the prefix still to take
  __shared__ int s_valid;    // keys > 0 in the row (capped)
  __shared__ K skey[kMaxK];
  __shared__ int64_t sidx[kMaxK];
  __shared__ int s_cnt;
  __shared__ int s_eqbase;
  const int64_t r = blockIdx.x / nseg, seg = blockIdx.x % nseg;
  const int64_t off = r * row_stride + seg * seg_len;
  const V *row = x + off;
  const int64_t n = min(seg_len, n_row - seg * seg_len);
  const int64_t o = (int64_t)blockIdx.x * k;
  // number of valid keys (capped at k): the answer holds min(k, valid) entries
  if (threadIdx.x == 0) s_valid = 0;
  __syncthreads();
  {
    int cnt = 0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) cnt += KO::key(row[i]) != 0;
    if (cnt) atomicAdd(&s_valid, cnt);
  }
  __syncthreads();
  const int take = s_valid < k ? s_valid : k;
  if (take == 0) {
    for (int i = threadIdx.x; i < k; i += blockDim.x) {
      idx_out[o + i] = -1;
      val_out[o + i] = (V)0;
    }
    if (threadIdx.x == 0) count_out[blockIdx.x] = 0;
    return;
  }
  // radix select of the take-th largest key
  if (threadIdx.x == 0) {
    s_prefix = 0;
    s_need = take;
  }
  __syncthreads();
  K mask = 0;
  for (int shift = KO::kBits - 8; shift >= 0; shift -= 8) {
    for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b] = 0;
    __syncthreads();
    const K prefix = s_prefix;
    // warp-aggregated increments: the keys of a row often share their high
    // bytes, so one atomic per distinct bin per warp instead of per key
    const int lane = threadIdx.x & 31;
    for (int64_t base = 0; base < n; base += blockDim.x) {
      const int64_t i = base + threadIdx.x;
      const K kk = i < n ? KO::key(row[i]) : (K)0;
      const bool hit = kk != 0 && (kk & mask) == prefix;
      const unsigned bin = hit ? (unsigned)((kk >> shift) & 0xFF) : 256u + (unsigned)lane;  // misses: unique keys
      const unsigned peers = __match_any_sync(0xffffffffu, bin);
      if (hit && lane == __ffs(peers) - 1) atomicAdd(&hist[bin], (unsigned)__popc(peers));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int need = s_need;
      int b = 255;
      for (; b > 0; --b) {
        if ((int)hist[b] >= need) break;
        need -= (int)hist[b];
      }
      s_prefix = prefix | ((K)b << shift);
      s_need = need;  // keys equal to the final prefix still to take
    }
    __syncthreads();
    mask |= (K)0xFF << shift;
  }
  const K thr = s_prefix;
  const int need_eq = s_need;
  // collection: every key above thr, and the need_eq lowest-index keys equal to it
  if (threadIdx.x == 0) {
    s_cnt = 0;
    s_eqbase = 0;
  }
  __syncthreads();
  __shared__ int wsum[kTThreads / 32];
  for (int64_t base = 0; base < n; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    const K kk = i < n ? KO::key(row[i]) : 0;
    if (kk > thr) {
      const int pos = atomicAdd(&s_cnt, 1);
      skey[pos] = kk;
      sidx[pos] = i;
    }
    // ties in index order: block-wide exclusive count of equal keys
    const int eq = (i < n && kk == thr) ? 1 : 0;
    const unsigned bal = __ballot_sync(0xffffffffu, eq);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) wsum[wid] = __popc(bal);
    __syncthreads();
    int before = s_eqbase;
    for (int w = 0; w < wid; ++w) before += wsum[w];
    before += __popc(bal & ((1u << lane) - 1u));
    if (eq && before < need_eq) {
      const int pos = take - need_eq + before;  // tie slots follow the `take - need_eq` larger keys
      skey[pos] = kk;
      sidx[pos] = i;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += wsum[w];
      s_eqbase += t;
    }
    __syncthreads();
    if (s_eqbase >= need_eq && s_cnt >= take - need_eq) break;  // uniform: shared values after a barrier
  }
  __syncthreads();
  // bitonic sort of take entries by (key desc, index asc), padded to a power of two
  int p2 = 1;
  while (p2 < take) p2 <<= 1;
  for (int i = take + threadIdx.x; i < p2; i += blockDim.x) {
    skey[i] = 0;
    sidx[i] = INT64_MAX;
  }
  __syncthreads();
  for (int size = 2; size <= p2; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < p2; i += blockDim.x) {
        const int j = i ^ stride;
        if (j > i) {
          const bool up = (i & size) == 0;  // this pair's half sorts "first before second"
          // "a before b": larger key, or equal key and smaller index
          const bool a_first = skey[i] > skey[j] || (skey[i] == skey[j] && sidx[i] < sidx[j]);
          if (a_first != up) {
            const K tk = skey[i];
            skey[i] = skey[j];
            skey[j] = tk;
            const int64_t ti = sidx[i];
            sidx[i] = sidx[j];
            sidx[j] = ti;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    if (i < take) {
      idx_out[o + i] = idx_map ? idx_map[off + sidx[i]] : seg * seg_len + sidx[i];
      val_out[o + i] = row[sidx[i]];
    } else {
      idx_out[o + i] = -1;
      val_out[o + i] = (V)0;
    }
  }
  if (threadIdx.x == 0) count_out[blockIdx.x] = take;
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
  const int64_t nseg = n > 2 * kSegLen ? ceil_div<int64_t>(n, kSegLen) : 1;
  cudaError_t e = dev_malloc_async((void **)&d_idx, sizeof(int64_t) * rows * k, s);
  if (e == cudaSuccess) e = dev_malloc_async((void **)&d_val, sizeof(V) * rows * k, s);
  if (e == cudaSuccess) e = dev_malloc_async((void **)&d_cnt, sizeof(int64_t) * rows, s);
  if (nseg > 1) {
    if (e == cudaSuccess) e = dev_malloc_async((void **)&c_idx, sizeof(int64_t) * rows * nseg * k, s);
    if (e == cudaSuccess) e = dev_malloc_async((void **)&c_val, sizeof(V) * rows * nseg * k, s);
    if (e == cudaSuccess) e = dev_malloc_async((void **)&c_cnt, sizeof(int64_t) * rows * nseg, s);
  }
  for (int64_t r0 = 0; r0 < rows && e == cudaSuccess; r0 += kRowsPerLaunch) {
    const int64_t nr = rows - r0 < kRowsPerLaunch ? rows - r0 : kRowsPerLaunch;
    if (nseg == 1) {
      topk_rows<V><<<(unsigned)nr, kTThreads, 0, s>>>(x + r0 * n, n, n, n, 1, (int)k, nullptr, d_idx + r0 * k,
                                                       d_val + r0 * k, d_cnt + r0);
    } else {
      const int64_t nc = nseg * k;  // candidates per row
      topk_rows<V><<<(unsigned)(nr * nseg), kTThreads, 0, s>>>(x + r0 * n, n, kSegLen, n, (int)nseg, (int)k, nullptr,
                                                                c_idx + r0 * nc, c_val + r0 * nc, c_cnt + r0 * nseg);
      topk_rows<V><<<(unsigned)nr, kTThreads, 0, s>>>(c_val + r0 * nc, nc, nc, nc, 1, (int)k, c_idx + r0 * nc,
                                                       d_idx + r0 * k, d_val + r0 * k, d_cnt + r0);
    }
    e = cudaGetLastError();
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
