// Row-tile GEMMs of the warm start's network on the 5th-generation tensor
// cores (tcgen05) with TMA-fed operands:
//
//   layer-2 forward   H2 = relu([H1 | A1] W2 + b2), u = H2 w3 + b3, w = exp(u)
//                     (M = n, K = 256, N = 128)
//   input gradient    [dH1 | dA1] = dH2 W2^T                 (M = n, K = 128, N = 256)
//
// A persistent CTA per SM walks 128-row tiles.  Warp 0 (one lane) streams the
// A operand through a ring of 64-column k-blocks with TMA (128-byte swizzle,
// rows past n read as zeros) after loading the CTA's whole B operand once;
// warp 1 allocates the tensor memory and (one lane) issues
// tcgen05.mma.cta_group::1.kind::f16 (BF16 x BF16 -> FP32, M = 128, N = the
// output width, K = 16 per instruction) into one of two accumulators, so the
// epilogue of tile i overlaps the loads and products of tile i + 1; warps
// 2..9 read the accumulator back with tcgen05.ld (each warp its 32-lane
// quarter of the rows and one half of the columns) and apply the epilogue.
// Stages, accumulators and the B operand are handed over with mbarriers;
// every wait gives up after about two seconds (globaltimer), sets the error
// flag, and the CTA winds down and frees its tensor memory, so a broken
// handshake ends the kernel instead of hanging it.
//
// Numerics: FP32 accumulation of BF16 products; the layer-2 head sums the
// row's 128 rounded activations times w3 in column order (each half in order,
// then half 0 + half 1), so results are deterministic.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <mutex>

#include "warm.cuh"
#include "warm_tc.cuh"

namespace gops {
namespace {

using bf16 = __nv_bfloat16;

constexpr int kTM = 128;            // rows per tile (the MMA's M)
constexpr int kKB = 64;             // columns per k-block: 64 BF16 = one 128-byte swizzled row
constexpr int kStages = 6;          // k-blocks of A in flight
constexpr int kEpiWarps = 8;        // two per 32-lane quarter of the accumulator
constexpr int kTcThreads = 64 + 32 * kEpiWarps;
constexpr uint32_t kABytes = kTM * 128;       // one k-block of A
constexpr unsigned long long kWaitNs = 2000000000ull;
constexpr int kBars = 2 * kStages + 8;        // mbarriers (8 bytes each)

// ---- PTX wrappers ----------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for the phase of `parity` to complete; false when the CTA is winding
// down (abort set) or after kWaitNs, in which case the error flag gets `code`.
__device__ __noinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort, int *err, int code) {
  unsigned long long t0 = 0;
  for (uint32_t i = 0;; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 255u) {
      if (*abort) return false;
      const unsigned long long t = globaltimer();
      if (t0 == 0) {
        t0 = t;
      } else if (t - t0 > kWaitNs) {
        *abort = 1;
        atomicExch(err, code);
        return false;
      }
    }
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major operand in 128-byte swizzled rows
// (TMA's SWIZZLE_128B layout), 8-row groups 1024 bytes apart.  Bits: start
// address >> 4 [0,14), leading-dimension byte offset >> 4 [16,30) (not used
// by swizzled K-major layouts), stride-dimension byte offset >> 4 [32,46),
// descriptor version 1 [46,48), swizzle mode 2 = 128-byte [61,64).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator [4,6) = 1, A and B
// BF16 [7,10) = [10,13) = 1, both K-major (bits 15, 16 = 0), N >> 3 at
// [17,23), M >> 4 at [24,29).
constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
// arrive on `bar` when every tcgen05.mma this thread issued so far has completed
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
        "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
        "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ---- the kernel ------------------------------------------------------------
// Y[row][y0 + c] for the CTA's output columns c < NB (y0 = blockIdx.y * NB) =
// sum over k < K of X[row][k] * Bt[y0 + c][k], X = [Xa | Xb] (Xa has ka
// columns; k-block j reads Xa when 64 j < ka, else Xb).
template <int K, int NB, int EPI>
__global__ void __launch_bounds__(kTcThreads, 1)
    tc_rows(const __grid_constant__ CUtensorMap map_xa, const __grid_constant__ CUtensorMap map_xb,
            const __grid_constant__ CUtensorMap map_bt, int ka, int64_t M, TcEpi e, int *err) {
  static_assert(K % kKB == 0 && NB % 32 == 0 && NB >= 32 && NB <= 256, "tile shape");
  constexpr int KBLK = K / kKB;
  constexpr uint32_t kBBlk = NB * 128;  // one k-block of B
  constexpr uint32_t kIdesc = idesc_bf16(kTM, NB);
  constexpr int kHalf = NB / 2;          // columns per epilogue warp
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char *sm = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
  unsigned char *sB = sm;
  unsigned char *sA = sB + KBLK * kBBlk;
  uint64_t *bars = reinterpret_cast<uint64_t *>(sA + kStages * kABytes);
  // full[s], empty[s], b_full, acc_full[2], acc_empty[2], head[2], drain
  const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * kStages, bfull = empty0 + 8 * kStages;
  const uint32_t accf0 = bfull + 8, acce0 = accf0 + 16, head0 = acce0 + 16, drain = head0 + 16;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + kBars);
  float *red = reinterpret_cast<float *>(tmem_slot + 4);  // [2 tiles][2 halves][kTM]
  __shared__ int s_abort;
  volatile int *abort = &s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t tiles = (M + kTM - 1) / kTM;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    mbar_init(bfull, 1);
    for (int a = 0; a < 2; ++a) {
      mbar_init(accf0 + 8 * a, 1);
      mbar_init(acce0 + 8 * a, kEpiWarps);
      mbar_init(head0 + 8 * a, kEpiWarps);
    }
    mbar_init(drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_abort = 0;
  }
  if (warp == 1) {  // two accumulators of NB FP32 columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2 * NB)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // B: the CTA's NB rows of Bt, every k-block, once
      mbar_expect_tx(bfull, KBLK * kBBlk);
      for (int j = 0; j < KBLK; ++j)
        tma_load_2d(smem_u32(sB + j * kBBlk), &map_bt, j * kKB, (int)blockIdx.y * NB, bfull);
      uint32_t it = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
        for (int j = 0; j < KBLK; ++j, ++it) {
          const uint32_t s = it % kStages, ph = (it / kStages) & 1u;
          if (!mbar_wait(empty0 + 8 * s, ph ^ 1u, abort, err, 1)) {
            ok = false;
            break;
          }
          mbar_expect_tx(full0 + 8 * s, kABytes);
          const int x = j * kKB;
          if (x < ka) tma_load_2d(smem_u32(sA + s * kABytes), &map_xa, x, (int)(t * kTM), full0 + 8 * s);
          else tma_load_2d(smem_u32(sA + s * kABytes), &map_xb, x - ka, (int)(t * kTM), full0 + 8 * s);
        }
      }
      // winding down early: let the copies already issued land before the CTA exits
      if (!ok) {
        for (uint32_t q = it > kStages ? it - kStages : 0; q < it; ++q) {
          const uint32_t s = q % kStages, ph = (q / kStages) & 1u;
          unsigned long long t0 = globaltimer();
          while (!mbar_try_wait(full0 + 8 * s, ph) && globaltimer() - t0 < kWaitNs) {
          }
        }
        unsigned long long t0 = globaltimer();
        while (!mbar_try_wait(bfull, 0) && globaltimer() - t0 < kWaitNs) {
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      bool ok = mbar_wait(bfull, 0, abort, err, 2);
      uint32_t it = 0, i = 0;
      for (int64_t t = blockIdx.x; t < tiles && ok; t += gridDim.x, ++i) {
        const uint32_t a = i & 1u, aph = (i >> 1) & 1u;
        if (!mbar_wait(acce0 + 8 * a, aph ^ 1u, abort, err, 3)) break;
        tc_fence_after();
        const uint32_t d = tmem + a * NB;
        for (int j = 0; j < KBLK; ++j, ++it) {
          const uint32_t s = it % kStages, ph = (it / kStages) & 1u;
          if (!mbar_wait(full0 + 8 * s, ph, abort, err, 4)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a_base = smem_u32(sA + s * kABytes), b_base = smem_u32(sB + j * kBBlk);
#pragma unroll
          for (int kk = 0; kk < kKB / 16; ++kk)  // 16 BF16 = 32 bytes per MMA along K
            umma_bf16(d, sdesc(a_base + 32 * kk), sdesc(b_base + 32 * kk), kIdesc, (j | kk) != 0);
          umma_commit(empty0 + 8 * s);  // the stage is free once these products are done
        }
        if (!ok) break;
        umma_commit(accf0 + 8 * a);
      }
      // every product issued has completed before the tensor memory is freed
      umma_commit(drain);
      const unsigned long long t0 = globaltimer();
      while (!mbar_try_wait(drain, 0) && globaltimer() - t0 < kWaitNs) {
      }
    }
    __syncwarp();
  } else {
    const int q = warp & 3;                   // TMEM lanes 32q .. 32q + 31: tile rows
    const int h = (warp - 2) / 4;             // column half
    const int rl = 32 * q + lane;             // this thread's row in the tile
    uint32_t i = 0;
    for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x, ++i) {
      const uint32_t a = i & 1u, aph = (i >> 1) & 1u;
      if (!mbar_wait(accf0 + 8 * a, aph, abort, err, 5)) break;
      tc_fence_after();
      const int64_t row = t * kTM + rl;
      const bool in = row < M;
      float hs = 0.f;
      const uint32_t tbase = tmem + ((uint32_t)(32 * q) << 16) + a * NB + h * kHalf;
#pragma unroll 1
      for (int c0 = 0; c0 < kHalf; c0 += 32) {
        uint32_t v[32];
        tmem_ld32(tbase + c0, v);
        const int col0 = h * kHalf + c0;
        uint32_t packed[16];
#pragma unroll
        for (int c = 0; c < 32; c += 2) {
          float f0 = __uint_as_float(v[c]), f1 = __uint_as_float(v[c + 1]);
          if constexpr (EPI == kTcLayer2) {
            f0 += __ldg(&e.bias[col0 + c]);
            f1 += __ldg(&e.bias[col0 + c + 1]);
          }
          if constexpr (EPI != kTcStore) {
            f0 = fmaxf(f0, 0.f);
            f1 = fmaxf(f1, 0.f);
          }
          const __nv_bfloat162 pv = __floats2bfloat162_rn(f0, f1);
          if constexpr (EPI == kTcLayer2) {  // the head reads the stored (rounded) activations
            const float2 r2 = __bfloat1622float2(pv);
            hs = fmaf(r2.x, __ldg(&e.head[col0 + c]), hs);
            hs = fmaf(r2.y, __ldg(&e.head[col0 + c + 1]), hs);
          }
          packed[c / 2] = *reinterpret_cast<const uint32_t *>(&pv);
        }
        if (in) {
          uint4 *dst = reinterpret_cast<uint4 *>(e.out + row * e.ld + (int64_t)blockIdx.y * NB + col0);
#pragma unroll
          for (int u = 0; u < 4; ++u)
            dst[u] = make_uint4(packed[4 * u], packed[4 * u + 1], packed[4 * u + 2], packed[4 * u + 3]);
        }
      }
      // the accumulator is read: the next tile but one may overwrite it
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acce0 + 8 * a);
      if constexpr (EPI == kTcLayer2) {
        // the two column halves' head sums meet in shared memory (buffer i & 1;
        // an mbarrier per buffer, one arrival per epilogue warp)
        float *rt = red + (i & 1u) * 2 * kTM;
        rt[h * kTM + rl] = hs;
        __syncwarp();
        if (lane == 0) mbar_arrive(head0 + 8 * a);
        if (!mbar_wait(head0 + 8 * a, aph, abort, err, 6)) break;
        if (h == 0 && in) {
          float u = (rt[rl] + rt[kTM + rl]) + __ldg(&e.head[NB]);
          u = fminf(fmaxf(u, -20.f), 20.f);
          e.w[row] = expf(u);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * NB) : "memory");
  }
}

template <int K, int NB>
constexpr size_t tc_smem() {
  return 1024 + (size_t)(K / kKB) * NB * 128 + (size_t)kStages * kABytes + 8 * kBars + 16 + sizeof(float) * 4 * kTM;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point, so that
// the library does not link the driver library itself (it loads on machines
// without a GPU driver; this path is only taken with a device).
PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 2-D BF16 tensor map of a row-major [rows][cols] array, boxes of 64 columns
// x box_rows rows, 128-byte swizzle; reads past the array give zeros.
Status make_map(CUtensorMap *map, const bf16 *base, int64_t rows, int cols, int box_rows) {
  if (cols % 8 != 0 || (reinterpret_cast<uintptr_t>(base) & 15u) != 0)
    return Status{GOPS_ERR_INTERNAL, "tensor map: rows must be 16-byte aligned"};
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)cols * sizeof(bf16)};
  const cuuint32_t box[2] = {(cuuint32_t)kKB, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const PFN_cuTensorMapEncodeTiled_v12000 encode = encode_tiled();
  if (!encode) return Status{GOPS_ERR_CUDA, "cuTensorMapEncodeTiled is not available"};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16 *>(base), dims,
                                            strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return Status{GOPS_ERR_CUDA, "cuTensorMapEncodeTiled failed"};
  return Status::ok();
}

template <int K, int NB, int EPI>
Status launch(Ctx *ctx, const bf16 *xa, int ka, const bf16 *xb, const bf16 *bt, int ntot, int64_t m,
              const TcEpi &e, int *err) {
  if (m <= 0) return Status::ok();
  if (ka % kKB != 0 || ka > K || ntot % NB != 0) return Status{GOPS_ERR_INTERNAL, "tc_rows: operand shape"};
  CUtensorMap ma, mb, mw;
  GOPS_TRY(make_map(&ma, xa, m, ka, kTM));
  GOPS_TRY(make_map(&mb, ka < K ? xb : xa, m, ka < K ? K - ka : ka, kTM));
  GOPS_TRY(make_map(&mw, bt, ntot, K, NB));
  constexpr size_t smem = tc_smem<K, NB>();
  static bool attr = false;  // per instantiation
  if (!attr) {
    GOPS_CUDA_TRY(cudaFuncSetAttribute(tc_rows<K, NB, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  const int64_t tiles = (m + kTM - 1) / kTM;
  dim3 grid((unsigned)std::min<int64_t>(tiles, ctx->num_sms), (unsigned)(ntot / NB));
  tc_rows<K, NB, EPI><<<grid, kTcThreads, smem, ctx->stream>>>(ma, mb, mw, ka, m, e, err);
  GOPS_CUDA_TRY(cudaGetLastError());
  return Status::ok();
}

}  // namespace

Status tc_layer2(Ctx *ctx, const bf16 *h1, const bf16 *a1, const bf16 *w2t, int64_t n, const TcEpi &e, int *err) {
  return launch<2 * kWH, kWH, kTcLayer2>(ctx, h1, kWH, a1, w2t, kWH, n, e, err);
}

Status tc_input_grad(Ctx *ctx, const bf16 *g2, const bf16 *w2, int64_t n, const TcEpi &e, int *err) {
  return launch<kWH, 2 * kWH, kTcStore>(ctx, g2, kWH, nullptr, w2, 2 * kWH, n, e, err);
}

}  // namespace gops

extern "C" int gops_debug_tc_gemm(gops_ctx *ctx, int mode, const void *xa, const void *xb, const void *bt, int64_t m,
                                  void *out, const float *bias, const float *head, float *w, int *err) {
  using namespace gops;
  if (!ctx) return GOPS_ERR_INVALID;
  Ctx &c = ctx->impl;
  if (m < 0 || !xa || !bt || !out || !err || (mode == 0 && (!xb || !bias || !head || !w)))
    return c.set(Status{GOPS_ERR_INVALID, "null argument"});
  cudaSetDevice(c.device);
  const auto *a = static_cast<const bf16 *>(xa), *b = static_cast<const bf16 *>(xb),
             *t = static_cast<const bf16 *>(bt);
  Status st;
  if (mode == 0) st = tc_layer2(&c, a, b, t, m, TcEpi{static_cast<bf16 *>(out), kWH, bias, head, w}, err);
  else if (mode == 1) st = tc_input_grad(&c, a, t, m, TcEpi{static_cast<bf16 *>(out), 2 * kWH, nullptr, nullptr, nullptr}, err);
  else st = Status{GOPS_ERR_INVALID, "mode must be 0 or 1"};
  if (st.code == GOPS_OK) {
    const cudaError_t e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) st = Status{GOPS_ERR_CUDA, cudaGetErrorString(e)};
  }
  return c.set(st);
}
