// Internal helpers shared by the libgops CUDA translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "gops.h"

namespace gops {

constexpr int kWarp = 32;

// ---------------------------------------------------------------------------
// Error plumbing: every entry point returns a gops status and leaves a message
// in the context (gops_last_error).
// ---------------------------------------------------------------------------
struct Status {
  int code = GOPS_OK;
  std::string msg;
  static Status ok() { return {}; }
};

#define GOPS_CUDA_TRY(expr)                                                      \
  do {                                                                           \
    cudaError_t _e = (expr);                                                     \
    if (_e != cudaSuccess) {                                                     \
      return ::gops::Status{_e == cudaErrorMemoryAllocation ? GOPS_ERR_OOM       \
                                                            : GOPS_ERR_CUDA,     \
                            std::string(#expr) + ": " + cudaGetErrorString(_e)}; \
    }                                                                            \
  } while (0)

#define GOPS_TRY(expr)                  \
  do {                                  \
    ::gops::Status _s = (expr);         \
    if (_s.code != GOPS_OK) return _s;  \
  } while (0)

// ---------------------------------------------------------------------------
// Double-float ("DF") arithmetic: a value is hi + lo with two FP32 words,
// about 48 significant bits, using only FP32 instructions (GB300 runs FP64 at
// a small fraction of its FP32 rate).  Error-free transforms after Dekker
// (1971) and Knuth (TAOCP vol. 2, 4.2.2): TwoSum, FastTwoSum, and TwoProd via
// fused multiply-add.
// ---------------------------------------------------------------------------
struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_make(float h) { return {h, 0.0f}; }

__device__ __forceinline__ df two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b|
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}

__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, e);
}

__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ df df_mul_f(df a, float b) {
  float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fmaf_rn(a.lo, b, e);
  return fast_two_sum(p, e);
}

__device__ __forceinline__ df df_mul(df a, df b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

// a / b for an FP32 divisor (exact remainder through fma).
__device__ __forceinline__ df df_div_f(df a, float b) {
  float q = __fdiv_rn(a.hi, b);
  float r = __fmaf_rn(-q, b, a.hi);
  r = __fadd_rn(r, a.lo);
  float q2 = __fdiv_rn(r, b);
  return fast_two_sum(q, q2);
}

__host__ __device__ inline df df_from_double(double x) {
  float h = (float)x;
  float l = (float)(x - (double)h);
  return {h, l};
}

__device__ __forceinline__ df shfl_xor_df(df v, int lane_mask, int width) {
  v.hi = __shfl_xor_sync(0xffffffffu, v.hi, lane_mask, width);
  v.lo = __shfl_xor_sync(0xffffffffu, v.lo, lane_mask, width);
  return v;
}

// ---------------------------------------------------------------------------
// Exact global sums in 64-bit fixed point.  A term x contributes
// round(x * 2^F); integer addition is associative, so per-thread, per-block
// and atomic accumulation give the same total in any order (deterministic),
// and the total is exact for the rounded terms.  F is chosen per solve so
// that every partial stays below 2^62 in magnitude.
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long fx_of(float x, float scale) {
  return __float2ll_rn(__fmul_rn(x, scale));  // power-of-two scale: exact product
}

__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ int warp_or(int v) {
  return __reduce_or_sync(0xffffffffu, (unsigned)v);
}

// ---------------------------------------------------------------------------
// Bulk asynchronous copies (TMA, non-tensor form) into shared memory, with
// mbarrier completion.  Addresses and sizes must be multiples of 16 bytes.
// Every wait is bounded: after kWaitLimit polls it gives up and returns false.
// ---------------------------------------------------------------------------
constexpr uint32_t kWaitLimit = 1u << 24;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (bulk copy) accesses.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;"
               ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
  return ok != 0;
}

// Bounded wait for the phase with the given parity to complete.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  for (uint32_t i = 0; i < kWaitLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Device memory.  Every allocation of the library is stream-ordered and comes
// from one pool per device that keeps freed memory for reuse (its release
// threshold is unlimited; gops_ctx_destroy trims what no live object holds).
// Re-mapping the ~3 GB that an upload and build of a 4 M-node, 65 M-edge graph
// allocate and free cost ~4 ms per upload with the default pool, which returns
// memory at every synchronisation.  cudaFree releases these allocations without
// synchronising (the caller has finished every access: each call of the
// library waits for its stream before it returns).
cudaMemPool_t library_pool(int device);  // nullptr: pool not available
void library_pool_trim(int device);
// Host-side fault injection for tests (gops_debug_fail_allocations_after):
// true when this allocation is to fail as if the device were out of memory.
bool alloc_fault_injected();
inline cudaError_t dev_malloc_async(void **p, size_t bytes, cudaStream_t s) {
  if (alloc_fault_injected()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  int d = 0;
  cudaError_t e = cudaGetDevice(&d);
  if (e != cudaSuccess) return e;
  cudaMemPool_t pool = library_pool(d);
  return pool ? cudaMallocFromPoolAsync(p, bytes, pool, s) : cudaMallocAsync(p, bytes, s);
}
template <typename T>
inline cudaError_t dev_malloc_async(T **p, size_t bytes, cudaStream_t s) {
  return dev_malloc_async(reinterpret_cast<void **>(p), bytes, s);
}

// Stream-ordered free that tolerates NULL (cudaFreeAsync(NULL) is not a no-op).
inline void free_async(void *p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

template <typename T>
__host__ __device__ inline T ceil_div(T a, T b) {
  return (a + b - 1) / b;
}

// CTAs for `work` items of `threads` each, at least 1 and at most `cap`
inline int blocks_for(int64_t work, int threads, int cap) {
  const int64_t b = (work + threads - 1) / threads;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace gops
