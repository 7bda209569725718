// Exclusive scan and stable LSD radix sort (see primitives.cuh).
#include "primitives.cuh"

namespace gops {
namespace {

constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

// Block-wide exclusive scan of one value per thread; returns the block total
// through *total.
template <typename T>
__device__ T block_exclusive_scan(T v, T *total) {
  __shared__ T warp_tot[kScanThreads / kWarp];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  T incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    T w = (lane < kScanThreads / kWarp) ? warp_tot[lane] : T(0);
    T wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    if (lane < kScanThreads / kWarp) warp_tot[lane] = wi - w;  // exclusive warp offsets
    if (lane == kScanThreads / kWarp - 1) warp_tot[kScanThreads / kWarp - 1] = wi - w, *total = wi;
  }
  __syncthreads();
  T r = warp_tot[wid] + incl - v;
  __syncthreads();
  return r;
}

template <typename T>
__global__ void scan_tile_sums(const T *in, int64_t n, T *tile_sums) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  T s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) s += in[base + i];
  __shared__ T tot;
  block_exclusive_scan<T>(s, &tot);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

template <typename T>
__global__ void scan_tiles(const T *in, T *out, int64_t n, const T *tile_offsets) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  T v[kScanItems];
  T s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = (base + i < n) ? in[base + i] : T(0);
    s += v[i];
  }
  __shared__ T tot;
  T run = block_exclusive_scan<T>(s, &tot) + (tile_offsets ? tile_offsets[blockIdx.x] : T(0));
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
}

template <typename T>
Status exclusive_scan(const T *in, T *out, int64_t n, cudaStream_t s) {
  if (n <= 0) return Status::ok();
  const int64_t tiles = ceil_div<int64_t>(n, kScanTile);
  if (tiles == 1) {
    scan_tiles<T><<<1, kScanThreads, 0, s>>>(in, out, n, nullptr);
    GOPS_CUDA_TRY(cudaGetLastError());
    return Status::ok();
  }
  T *sums = nullptr;
  GOPS_CUDA_TRY(dev_malloc_async((void **)&sums, sizeof(T) * tiles, s));
  scan_tile_sums<T><<<(unsigned)tiles, kScanThreads, 0, s>>>(in, n, sums);
  Status st = exclusive_scan<T>(sums, sums, tiles, s);
  if (st.code == GOPS_OK) {
    scan_tiles<T><<<(unsigned)tiles, kScanThreads, 0, s>>>(in, out, n, sums);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) st = Status{GOPS_ERR_CUDA, std::string("scan: ") + cudaGetErrorString(e)};
  }
  free_async(sums, s);
  return st;
}

// ---------------------------------------------------------------------------
// Radix sort: 8-bit digits, tiles of 4096 items (8 warps x 512 consecutive
// items each).  Per pass: (1) per-tile digit histogram, (2) exclusive scan of
// the histogram in digit-major order, (3) stable scatter.  Inside a tile the
// rank of an item among equal digits comes from __match_any_sync within a
// 32-item chunk plus warp-private running counters, so the order of equal keys
// is preserved exactly.
// ---------------------------------------------------------------------------
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / kWarp;
constexpr int kPerWarp = 512;
constexpr int kSortTile = kSortWarps * kPerWarp;
constexpr int kRadix = 256;
static_assert(kSortThreads == kRadix, "the downsweep gives each thread one digit");

// Per tile: the count of every digit, in per-warp counters (a skewed digit's
// additions spread over eight addresses), from 16-byte loads of a full tile.
__global__ void radix_upsweep(const uint32_t *keys, int64_t n, int shift, uint32_t *hist,
                              int64_t tiles, int vec) {
  __shared__ uint32_t wc[kSortWarps][kRadix];
  for (int i = threadIdx.x; i < kSortWarps * kRadix; i += kSortThreads) (&wc[0][0])[i] = 0;
  __syncthreads();
  const int w = threadIdx.x >> 5;
  const int64_t base = (int64_t)blockIdx.x * kSortTile;
  if (vec && base + kSortTile <= n) {
    constexpr int kQuads = kSortTile / (4 * kSortThreads);
    uint4 q[kQuads];
#pragma unroll
    for (int j = 0; j < kQuads; ++j) q[j] = __ldg(reinterpret_cast<const uint4 *>(keys + base) + threadIdx.x + j * kSortThreads);
#pragma unroll
    for (int j = 0; j < kQuads; ++j) {
      atomicAdd(&wc[w][(q[j].x >> shift) & 0xFF], 1u);
      atomicAdd(&wc[w][(q[j].y >> shift) & 0xFF], 1u);
      atomicAdd(&wc[w][(q[j].z >> shift) & 0xFF], 1u);
      atomicAdd(&wc[w][(q[j].w >> shift) & 0xFF], 1u);
    }
  } else {
    for (int i = threadIdx.x; i < kSortTile; i += kSortThreads) {
      const int64_t idx = base + i;
      if (idx < n) atomicAdd(&wc[w][(keys[idx] >> shift) & 0xFF], 1u);
    }
  }
  __syncthreads();
  const int d = threadIdx.x;  // kSortThreads == kRadix
  uint32_t t = 0;
#pragma unroll
  for (int ww = 0; ww < kSortWarps; ++ww) t += wc[ww][d];
  hist[(int64_t)d * tiles + blockIdx.x] = t;
}

// Per tile: (a) warp-private digit counts (the tile's keys stay in
// registers), (b) tile-local start of every (warp, digit) and the offset from
// tile-local to global position per digit, (c) stable scatter into shared
// memory in digit order, (d) coalesced copy-out: consecutive threads write
// consecutive positions of a digit's run.
// vals == nullptr: the value of item idx is idx.
__global__ void __launch_bounds__(kSortThreads, 3) radix_downsweep(const uint32_t *keys, const uint32_t *vals,
                                                                uint32_t *okeys, uint32_t *ovals, int64_t n,
                                                                int shift, const uint32_t *offs, int64_t tiles) {
  constexpr int kChunks = kPerWarp / kWarp;
  __shared__ uint32_t wcnt[kSortWarps][kRadix];
  __shared__ uint32_t skeys[kSortTile];
  __shared__ uint32_t svals[kSortTile];
  __shared__ uint32_t gdelta[kRadix];  // global - tile-local position (mod 2^32)
  __shared__ uint32_t wsum[kSortWarps];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < kSortWarps * kRadix; i += kSortThreads) (&wcnt[0][0])[i] = 0;
  __syncthreads();
  const int64_t tbase = (int64_t)blockIdx.x * kSortTile;
  const int64_t wbase = tbase + (int64_t)w * kPerWarp;
  const unsigned lt_mask = (1u << lane) - 1u;
  uint32_t k[kChunks], v[kChunks];
  // (a) all of the warp's key loads go out before the digit counting, and the
  // value loads after it (in flight during (b)), so that their latencies
  // overlap: the counting's warp barriers would otherwise keep one chunk's
  // load in flight at a time
#pragma unroll
  for (int c = 0; c < kChunks; ++c) {
    const int64_t idx = wbase + c * kWarp + lane;
    k[c] = idx < n ? __ldg(keys + idx) : 0u;
  }
#pragma unroll
  for (int c = 0; c < kChunks; ++c) {
    const int64_t idx = wbase + c * kWarp + lane;
    const bool valid = idx < n;
    const unsigned dig = valid ? ((k[c] >> shift) & 0xFF) : 0x100u;
    const unsigned peers = __match_any_sync(0xffffffffu, dig);  // same digit in the 32-item chunk
    if (valid && lane == __ffs(peers) - 1) wcnt[w][dig] += __popc(peers);
    __syncwarp();
  }
#pragma unroll
  for (int c = 0; c < kChunks; ++c) {
    const int64_t idx = wbase + c * kWarp + lane;
    v[c] = vals ? (idx < n ? __ldg(vals + idx) : 0u) : (uint32_t)idx;  // no vals: the input position
  }
  __syncthreads();
  // (b) thread d owns digit d (kSortThreads == kRadix)
  {
    const int d = threadIdx.x;
    uint32_t tot = 0;
#pragma unroll
    for (int ww = 0; ww < kSortWarps; ++ww) {
      const uint32_t c = wcnt[ww][d];
      wcnt[ww][d] = tot;
      tot += c;
    }
    uint32_t incl = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    uint32_t loc = incl - tot;
    for (int ww = 0; ww < w; ++ww) loc += wsum[ww];
#pragma unroll
    for (int ww = 0; ww < kSortWarps; ++ww) wcnt[ww][d] += loc;
    gdelta[d] = offs[(int64_t)d * tiles + blockIdx.x] - loc;
  }
  __syncthreads();
  // (c) the peers are found again (cheaper than keeping 16 masks live)
#pragma unroll
  for (int c = 0; c < kChunks; ++c) {
    const int64_t idx = wbase + c * kWarp + lane;
    const bool valid = idx < n;
    const unsigned dig = valid ? ((k[c] >> shift) & 0xFF) : 0x100u;
    const unsigned peers = __match_any_sync(0xffffffffu, dig);
    const uint32_t pos = valid ? wcnt[w][dig] + __popc(peers & lt_mask) : 0u;
    __syncwarp();
    if (valid) {
      skeys[pos] = k[c];
      svals[pos] = v[c];
      if (lane == __ffs(peers) - 1) wcnt[w][dig] += __popc(peers);
    }
    __syncwarp();
  }
  __syncthreads();
  // (d)
  const int cnt = (int)(n - tbase < (int64_t)kSortTile ? n - tbase : (int64_t)kSortTile);
  for (int i = threadIdx.x; i < cnt; i += kSortThreads) {
    const uint32_t kk = skeys[i];
    const uint32_t pos = (uint32_t)i + gdelta[(kk >> shift) & 0xFF];
    okeys[pos] = kk;
    ovals[pos] = svals[i];
  }
}

}  // namespace

Status exclusive_scan_i64(const int64_t *in, int64_t *out, int64_t n, cudaStream_t s) {
  return exclusive_scan<long long>((const long long *)in, (long long *)out, n, s);
}

Status exclusive_scan_u32(const uint32_t *in, uint32_t *out, int64_t n, cudaStream_t s) {
  return exclusive_scan<uint32_t>(in, out, n, s);
}

namespace {

__global__ void iota_fill(uint32_t *v, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] = (uint32_t)i;
}

// keys_in/vals_in: the first pass's input (vals_in nullptr: positions);
// later passes ping-pong between (keys, vals) and (keys_alt, vals_alt).
Status radix_sort_impl(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys, uint32_t *vals,
                       uint32_t *keys_alt, uint32_t *vals_alt, int64_t n, int key_bits, bool *result_in_alt,
                       cudaStream_t s) {
  *result_in_alt = false;
  if (n <= 1 || key_bits <= 0) {  // already sorted: the input into (keys, vals)
    if (n > 0 && keys_in != keys)
      GOPS_CUDA_TRY(cudaMemcpyAsync(keys, keys_in, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s));
    if (n > 0 && !vals_in) {
      iota_fill<<<1, 256, 0, s>>>(vals, n);
      GOPS_CUDA_TRY(cudaGetLastError());
    }
    return Status::ok();
  }
  if (n >= (int64_t)UINT32_MAX) return Status{GOPS_ERR_INVALID, "radix sort: too many items"};
  const int64_t tiles = ceil_div<int64_t>(n, kSortTile);
  uint32_t *hist = nullptr;
  GOPS_CUDA_TRY(dev_malloc_async((void **)&hist, sizeof(uint32_t) * tiles * kRadix, s));
  uint32_t *bk[2] = {keys, keys_alt}, *bv[2] = {vals, vals_alt};
  int cur = 0;  // the buffer pair the next pass does not write
  const uint32_t *k_in = keys_in, *v_in = vals_in;
  Status st;
  for (int shift = 0; shift < key_bits; shift += 8) {
    const int vec = (reinterpret_cast<uintptr_t>(k_in) & 15) == 0;
    radix_upsweep<<<(unsigned)tiles, kSortThreads, 0, s>>>(k_in, n, shift, hist, tiles, vec);
    st = exclusive_scan_u32(hist, hist, tiles * kRadix, s);
    if (st.code != GOPS_OK) break;
    radix_downsweep<<<(unsigned)tiles, kSortThreads, 0, s>>>(k_in, v_in, bk[cur ^ 1], bv[cur ^ 1], n, shift,
                                                             hist, tiles);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      st = Status{GOPS_ERR_CUDA, std::string("radix sort: ") + cudaGetErrorString(e)};
      break;
    }
    cur ^= 1;
    k_in = bk[cur];
    v_in = bv[cur];
  }
  *result_in_alt = cur == 1;
  free_async(hist, s);
  return st;
}

}  // namespace

Status radix_sort_pairs_u32(uint32_t *keys, uint32_t *vals, uint32_t *keys_alt,
                            uint32_t *vals_alt, int64_t n, int key_bits,
                            bool *result_in_alt, cudaStream_t s) {
  return radix_sort_impl(keys, vals, keys, vals, keys_alt, vals_alt, n, key_bits, result_in_alt, s);
}

Status radix_sort_index_u32(const uint32_t *keys_in, uint32_t *keys, uint32_t *vals, uint32_t *keys_alt,
                            uint32_t *vals_alt, int64_t n, int key_bits, bool *result_in_alt,
                            cudaStream_t s) {
  return radix_sort_impl(keys_in, nullptr, keys, vals, keys_alt, vals_alt, n, key_bits, result_in_alt, s);
}

}  // namespace gops
