// The warm start's message-passing network (include/gops.h, gops_warm_*):
//
//   H1 = relu([x, mean_in x, 1] W1)                 (n x 48) . (48 x 128)
//   A1 = mean_in H1                                 over the in-edges
//   H2 = relu([H1, A1] W2 + b2)                     (n x 256) . (256 x 128)
//   u  = H2 w3 + b3,  w = exp(u)                    per-node weight
//
// Activations and the GEMM operands are BF16; every product accumulates in
// FP32 on the tensor cores.  At these shapes (K, N <= 256, M = n) the GEMMs
// move far more bytes than they multiply, so they are bound by HBM, not by
// the tensor pipe.  The two large row-tile GEMMs -- layer 2 (K = 256, with
// the bias, ReLU and head fused) and the input gradient dX = dH2 W2^T (N =
// 256) -- run on tcgen05 with TMA-fed operands (warm_tc.cu).  Layer 1 (K = 48,
// not a multiple of the 64-column swizzled k-block) and the weight gradients
// (dW = X^T dY, a reduction over the rows with per-CTA partials summed in a
// fixed order, so gradients are bit-reproducible) use mma.sync m16n8k16.
#include <cmath>
#include <vector>

#include "warm.cuh"
#include "warm_tc.cuh"

namespace gops {

namespace {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t ld_pair(const bf16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

constexpr int kBM = 64;    // rows per tile (row-tile GEMM)
constexpr int kBN = 128;   // output columns per CTA
constexpr int kGT = 256;   // threads per GEMM CTA (8 warps: 2 along M x 4 along N)

// out[M x 128-tile] = relu([Xa | Xb] (M x K) . Bt^T) (BF16, row stride ld),
// Bt = [Ntot][K] row-major (the B operand in the mma "col" layout).
// blockIdx.y selects the 128-column tile.  Persistent over row tiles; Bt's
// tile is staged once per CTA.  Layer 1 (K = 48).
template <int K>
__global__ void __launch_bounds__(kGT) gemm_rows(const bf16 *__restrict__ xa, int ka, const bf16 *__restrict__ xb,
                                                 const bf16 *__restrict__ bt, int64_t M, bf16 *__restrict__ out,
                                                 int ld) {
  constexpr int LD = K + 8;  // padded row (bf16): conflict-free fragment loads
  extern __shared__ __align__(16) unsigned char smem_raw[];
  bf16 *Bs = reinterpret_cast<bf16 *>(smem_raw);  // [kBN][LD]
  bf16 *Xs = Bs + kBN * LD;                       // [kBM][LD]
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int wm = wid & 1, wn = wid >> 1;
  const int g = lane >> 2, t4 = lane & 3;
  const int nt = blockIdx.y;
  const int kb = K - ka;
  // stage this CTA's 128 rows of Bt
  for (int i = tid; i < kBN * (K / 8); i += kGT) {
    const int r = i / (K / 8), c8 = (i % (K / 8)) * 8;
    *reinterpret_cast<uint4 *>(&Bs[r * LD + c8]) =
        *reinterpret_cast<const uint4 *>(&bt[(int64_t)(nt * kBN + r) * K + c8]);
  }
  const int64_t tiles = (M + kBM - 1) / kBM;
  for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int64_t row0 = tile * kBM;
    __syncthreads();  // Bs staged / previous tile's Xs consumed
    for (int i = tid; i < kBM * (K / 8); i += kGT) {
      const int r = i / (K / 8), c8 = (i % (K / 8)) * 8;
      const int64_t row = row0 + r;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (row < M)
        v = c8 < ka ? *reinterpret_cast<const uint4 *>(&xa[row * ka + c8])
                    : *reinterpret_cast<const uint4 *>(&xb[row * kb + (c8 - ka)]);
      *reinterpret_cast<uint4 *>(&Xs[r * LD + c8]) = v;
    }
    __syncthreads();
    float acc[2][4][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[a][b][q] = 0.f;
#pragma unroll 4
    for (int k0 = 0; k0 < K; k0 += 16) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        const bf16 *base = &Xs[(wm * 32 + a * 16 + g) * LD + k0 + 2 * t4];
        af[a][0] = ld_pair(base);
        af[a][1] = ld_pair(base + 8 * LD);
        af[a][2] = ld_pair(base + 8);
        af[a][3] = ld_pair(base + 8 * LD + 8);
      }
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const bf16 *base = &Bs[(wn * 32 + b * 8 + g) * LD + k0 + 2 * t4];
        bfr[b][0] = ld_pair(base);
        bfr[b][1] = ld_pair(base + 8);
      }
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) mma_bf16(acc[a][b], af[a], bfr[b]);
    }
    // epilogue: element (row, col) of acc[a][b][q]:
    //   row = wm*32 + a*16 + g + (q >= 2 ? 8 : 0), col = wn*32 + b*8 + 2*t4 + (q & 1)
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int hq = 0; hq < 2; ++hq) {
          const int rl = wm * 32 + a * 16 + g + hq * 8;
          const int col = wn * 32 + b * 8 + 2 * t4;
          const int64_t row = row0 + rl;
          const __nv_bfloat162 pv =
              __floats2bfloat162_rn(fmaxf(acc[a][b][hq * 2], 0.f), fmaxf(acc[a][b][hq * 2 + 1], 0.f));
          if (row < M) *reinterpret_cast<__nv_bfloat162 *>(&out[row * ld + (int64_t)nt * kBN + col]) = pv;
        }
  }
}

constexpr int kRC = 64;  // rows per chunk of the reduction GEMM
constexpr int kKT = 64;  // K rows of the output per CTA

// part[blockIdx.x][k][n] = sum over this CTA's slab of rows of X[row][k] D[row][n]
// for k in the CTA's K tile (blockIdx.y), n in [0, 128).  X = [Xa | Xb].
template <int K>
__global__ void __launch_bounds__(kGT) gemm_reduce(const bf16 *__restrict__ xa, int ka, const bf16 *__restrict__ xb,
                                                   const bf16 *__restrict__ d, int64_t M, int64_t slab,
                                                   float *__restrict__ part) {
  constexpr int LD = kRC + 8;
  __shared__ __align__(16) bf16 Xt[kKT][LD];   // Xt[k][i]
  __shared__ __align__(16) bf16 Dt[kBN][LD];   // Dt[n][i]
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int wm = wid & 1, wn = wid >> 1;
  const int g = lane >> 2, t4 = lane & 3;
  const int kt0 = blockIdx.y * kKT;
  const int kb = K - ka;
  const int64_t r0 = (int64_t)blockIdx.x * slab, r1 = min(M, r0 + slab);
  float acc[2][4][4];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[a][b][q] = 0.f;
  for (int64_t c0 = r0; c0 < r1; c0 += kRC) {
    __syncthreads();
    // X chunk: kRC rows x kKT columns, transposed into Xt
    for (int i = tid; i < kRC * (kKT / 2); i += kGT) {
      const int r = i / (kKT / 2), k2 = (i % (kKT / 2)) * 2;
      const int64_t row = c0 + r;
      const int k = kt0 + k2;
      __nv_bfloat162 v = __floats2bfloat162_rn(0.f, 0.f);
      if (row < r1 && k < K)
        v = k < ka ? *reinterpret_cast<const __nv_bfloat162 *>(&xa[row * ka + k])
                   : *reinterpret_cast<const __nv_bfloat162 *>(&xb[row * kb + (k - ka)]);
      Xt[k2][r] = v.x;
      Xt[k2 + 1][r] = v.y;
    }
    for (int i = tid; i < kRC * (kBN / 2); i += kGT) {
      const int r = i / (kBN / 2), n2 = (i % (kBN / 2)) * 2;
      const int64_t row = c0 + r;
      __nv_bfloat162 v = __floats2bfloat162_rn(0.f, 0.f);
      if (row < r1) v = *reinterpret_cast<const __nv_bfloat162 *>(&d[row * kBN + n2]);
      Dt[n2][r] = v.x;
      Dt[n2 + 1][r] = v.y;
    }
    __syncthreads();
#pragma unroll
    for (int k0 = 0; k0 < kRC; k0 += 16) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        const bf16 *base = &Xt[wm * 32 + a * 16 + g][k0 + 2 * t4];
        af[a][0] = ld_pair(base);
        af[a][1] = ld_pair(base + 8 * LD);
        af[a][2] = ld_pair(base + 8);
        af[a][3] = ld_pair(base + 8 * LD + 8);
      }
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const bf16 *base = &Dt[wn * 32 + b * 8 + g][k0 + 2 * t4];
        bfr[b][0] = ld_pair(base);
        bfr[b][1] = ld_pair(base + 8);
      }
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) mma_bf16(acc[a][b], af[a], bfr[b]);
    }
  }
  float *out = part + (int64_t)blockIdx.x * K * kBN;
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int hq = 0; hq < 2; ++hq) {
        const int k = kt0 + wm * 32 + a * 16 + g + hq * 8;
        const int col = wn * 32 + b * 8 + 2 * t4;
        if (k < K) {
          out[(int64_t)k * kBN + col] = acc[a][b][hq * 2];
          out[(int64_t)k * kBN + col + 1] = acc[a][b][hq * 2 + 1];
        }
      }
}

// dst[i] = sum over the `nparts` partial arrays (stride `stride`) of entry i, in order
__global__ void sum_parts(const float *__restrict__ part, int64_t nparts, int64_t stride, int64_t count,
                          float *__restrict__ dst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int64_t q = 0; q < nparts; ++q) s += part[q * stride + i];
    dst[i] = s;
  }
}

// out[v][:] = inv_in[v] * sum over in-edges (u -> v) of h[u][:] (128 BF16
// columns; a warp per node, four columns per lane, FP32 sums in edge order)
__global__ void agg_in_128(const int64_t *__restrict__ rp, const int32_t *__restrict__ col,
                           const float *__restrict__ inv, const bf16 *__restrict__ h, int64_t n,
                           bf16 *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t v = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); v < n; v += nw) {
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    for (int64_t e = rp[v]; e < rp[v + 1]; ++e) {
      const int64_t u = col[e];
      const uint2 q = *reinterpret_cast<const uint2 *>(&h[u * kWH + lane * 4]);
      const float2 f0 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&q.x));
      const float2 f1 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&q.y));
      s0 += f0.x; s1 += f0.y; s2 += f1.x; s3 += f1.y;
    }
    const float iv = inv[v];
    const __nv_bfloat162 o0 = __floats2bfloat162_rn(s0 * iv, s1 * iv);
    const __nv_bfloat162 o1 = __floats2bfloat162_rn(s2 * iv, s3 * iv);
    uint2 q;
    q.x = *reinterpret_cast<const uint32_t *>(&o0);
    q.y = *reinterpret_cast<const uint32_t *>(&o1);
    *reinterpret_cast<uint2 *>(&out[v * kWH + lane * 4]) = q;
  }
}

// cw[c] = sum of w over the members of cluster c (a warp per cluster, fixed order)
__global__ void cluster_sums(const int32_t *__restrict__ members, const int32_t *__restrict__ off, int r,
                             const float *__restrict__ w, float *__restrict__ cw) {
  const int lane = threadIdx.x & 31;
  for (int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < r; c += gridDim.x * (blockDim.x >> 5)) {
    float s = 0.f;
    for (int i = off[c] + lane; i < off[c + 1]; i += 32) s += w[members[i]];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) cw[c] = s;
  }
}

// dH2 = du * w3 * [H2 > 0] (BF16), and per-block partial sums of db2
// (sum_i dH2), dw3 (sum_i du_i H2_i) and db3 (sum_i du_i).  Thread t owns
// column t & 127 of every other row.  A node whose u was clamped passes no
// gradient (its du is zeroed by the caller).
constexpr int kHeadRows = 512;  // rows per block
__global__ void __launch_bounds__(256) head_backward(const float *__restrict__ du, const bf16 *__restrict__ h2,
                                                     const float *__restrict__ w3, int64_t n, bf16 *__restrict__ g2,
                                                     float *__restrict__ part) {
  __shared__ float sb[2][kWH], sw[2][kWH], s3[2];
  const int k = threadIdx.x & (kWH - 1), half = threadIdx.x >> 7;
  const int64_t r0 = (int64_t)blockIdx.x * kHeadRows, r1 = min(n, r0 + kHeadRows);
  const float wk = w3[k];
  float db2 = 0.f, dw3 = 0.f, db3 = 0.f;
  for (int64_t i = r0 + half; i < r1; i += 2) {
    const float d = du[i];
    const float h = __bfloat162float(h2[i * kWH + k]);
    const float gv = h > 0.f ? d * wk : 0.f;
    g2[i * kWH + k] = __float2bfloat16_rn(gv);
    db2 += gv;
    dw3 = fmaf(d, h, dw3);
    db3 += d;
  }
  sb[half][k] = db2;
  sw[half][k] = dw3;
  if (k == 0) s3[half] = db3;
  __syncthreads();
  float *out = part + (int64_t)blockIdx.x * (2 * kWH + 1);
  if (threadIdx.x < kWH) {
    out[k] = sb[0][k] + sb[1][k];
    out[kWH + k] = sw[0][k] + sw[1][k];
    if (k == 0) out[2 * kWH] = s3[0] + s3[1];
  }
}

// dH1[u] = (gx[u][0:128] + sum over out-edges (u -> v) of gx[v][128:256] / indeg(v)) * [H1 > 0]
__global__ void h1_backward(const int64_t *__restrict__ rp, const int32_t *__restrict__ col,
                            const float *__restrict__ inv_in, const bf16 *__restrict__ gx,
                            const bf16 *__restrict__ h1, int64_t n, bf16 *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t u = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); u < n; u += nw) {
    float s[4] = {0.f, 0.f, 0.f, 0.f};
    for (int64_t e = rp[u]; e < rp[u + 1]; ++e) {
      const int64_t v = col[e];
      const float iv = inv_in[v];
      const uint2 q = *reinterpret_cast<const uint2 *>(&gx[v * 2 * kWH + kWH + lane * 4]);
      const float2 f0 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&q.x));
      const float2 f1 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&q.y));
      s[0] = fmaf(f0.x, iv, s[0]); s[1] = fmaf(f0.y, iv, s[1]);
      s[2] = fmaf(f1.x, iv, s[2]); s[3] = fmaf(f1.y, iv, s[3]);
    }
    float o[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float direct = __bfloat162float(gx[u * 2 * kWH + lane * 4 + j]);
      const float h = __bfloat162float(h1[u * kWH + lane * 4 + j]);
      o[j] = h > 0.f ? direct + s[j] : 0.f;
    }
    const __nv_bfloat162 o0 = __floats2bfloat162_rn(o[0], o[1]);
    const __nv_bfloat162 o1 = __floats2bfloat162_rn(o[2], o[3]);
    uint2 q;
    q.x = *reinterpret_cast<const uint32_t *>(&o0);
    q.y = *reinterpret_cast<const uint32_t *>(&o1);
    *reinterpret_cast<uint2 *>(&out[u * kWH + lane * 4]) = q;
  }
}

// BF16 operand copies of the FP32 master weights
__global__ void refresh_bf16(const float *__restrict__ p, bf16 *__restrict__ w1t, bf16 *__restrict__ w2t,
                             bf16 *__restrict__ w2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kWIn * kWH) {  // W1 [k][n] -> w1t [n][k]
    const int k = i / kWH, nn = i % kWH;
    w1t[nn * kWIn + k] = __float2bfloat16_rn(p[kPW1 + i]);
  }
  if (i < 2 * kWH * kWH) {  // W2 [k][n] -> w2t [n][k] and w2 [k][n]
    const int k = i / kWH, nn = i % kWH;
    const bf16 v = __float2bfloat16_rn(p[kPW2 + i]);
    w2t[nn * 2 * kWH + k] = v;
    w2[i] = v;
  }
}

// Adam (Kingma & Ba, 2015) with bias correction
__global__ void adam_step(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                          float *__restrict__ v, int count, float lr, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gi = g[i];
  const float mi = 0.9f * m[i] + 0.1f * gi;
  const float vi = 0.999f * v[i] + 0.001f * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
}

uint64_t mix64(uint64_t z) {  // SplitMix64 finaliser (Steele, Lea, Flood 2014)
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

int gemm_ctas(const WarmModel &w, int64_t rows) {
  const int64_t tiles = (rows + kBM - 1) / kBM;
  return (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)w.ctx->num_sms * 2));
}

template <int K>
Status launch_rows(WarmModel &w, const bf16 *xa, int ka, const bf16 *xb, const bf16 *bt, int ntiles, bf16 *out,
                   int ld) {
  const size_t smem = sizeof(bf16) * (size_t)(kBN + kBM) * (K + 8);
  static bool attr = false;  // per instantiation
  if (!attr) {
    GOPS_CUDA_TRY(cudaFuncSetAttribute(gemm_rows<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  dim3 grid(gemm_ctas(w, w.n), ntiles);
  gemm_rows<K><<<grid, kGT, smem, w.ctx->stream>>>(xa, ka, xb, bt, w.n, out, ld);
  GOPS_CUDA_TRY(cudaGetLastError());
  return Status::ok();
}

template <int K>
Status launch_reduce(WarmModel &w, const bf16 *xa, int ka, const bf16 *xb, const bf16 *d, float *dst) {
  const int64_t slabs = std::max<int64_t>(1, std::min<int64_t>((w.n + kRC - 1) / kRC, (int64_t)w.ctx->num_sms * 2));
  const int64_t slab = ((w.n + slabs - 1) / slabs + kRC - 1) / kRC * kRC;
  const int64_t nslab = (w.n + slab - 1) / slab;
  dim3 grid((unsigned)std::max<int64_t>(nslab, 1), (K + kKT - 1) / kKT);
  if (nslab * K * kBN > w.part_cap) return Status{GOPS_ERR_INTERNAL, "warm start: partial buffer too small"};
  gemm_reduce<K><<<grid, kGT, 0, w.ctx->stream>>>(xa, ka, xb, d, w.n, slab, w.part);
  GOPS_CUDA_TRY(cudaGetLastError());
  sum_parts<<<blocks_for(K * kBN, 256, 1024), 256, 0, w.ctx->stream>>>(w.part, std::max<int64_t>(nslab, 1),
                                                                      (int64_t)K * kBN, (int64_t)K * kBN, dst);
  GOPS_CUDA_TRY(cudaGetLastError());
  return Status::ok();
}

}  // namespace

Status nn_alloc(WarmModel &w) {
  const int64_t n = std::max<int64_t>(w.n, 1);
  GOPS_CUDA_TRY(cudaMalloc(&w.params, sizeof(float) * kPCount));
  GOPS_CUDA_TRY(cudaMalloc(&w.adam_m, sizeof(float) * kPCount));
  GOPS_CUDA_TRY(cudaMalloc(&w.adam_v, sizeof(float) * kPCount));
  GOPS_CUDA_TRY(cudaMalloc(&w.grad, sizeof(float) * kPCount));
  GOPS_CUDA_TRY(cudaMalloc(&w.w1t, sizeof(bf16) * kWIn * kWH));
  GOPS_CUDA_TRY(cudaMalloc(&w.w2t, sizeof(bf16) * 2 * kWH * kWH));
  GOPS_CUDA_TRY(cudaMalloc(&w.w2, sizeof(bf16) * 2 * kWH * kWH));
  GOPS_CUDA_TRY(cudaMalloc(&w.h1, sizeof(bf16) * n * kWH));
  GOPS_CUDA_TRY(cudaMalloc(&w.a1, sizeof(bf16) * n * kWH));
  GOPS_CUDA_TRY(cudaMalloc(&w.h2, sizeof(bf16) * n * kWH));
  GOPS_CUDA_TRY(cudaMalloc(&w.g2, sizeof(bf16) * n * kWH));
  GOPS_CUDA_TRY(cudaMalloc(&w.gx, sizeof(bf16) * n * 2 * kWH));
  GOPS_CUDA_TRY(cudaMalloc(&w.w, sizeof(float) * n));
  GOPS_CUDA_TRY(cudaMalloc(&w.du, sizeof(float) * n));
  GOPS_CUDA_TRY(cudaMalloc(&w.cw, sizeof(float) * kWMaxClusters));
  const int64_t heads = (n + kHeadRows - 1) / kHeadRows;
  w.part_cap = std::max<int64_t>((int64_t)w.ctx->num_sms * 2 * 2 * kWH * kBN, heads * (2 * kWH + 1));
  GOPS_CUDA_TRY(cudaMalloc(&w.part, sizeof(float) * w.part_cap));
  GOPS_CUDA_TRY(cudaHostAlloc(&w.tc_err_h, sizeof(int), cudaHostAllocMapped));
  *w.tc_err_h = 0;
  GOPS_CUDA_TRY(cudaHostGetDevicePointer(&w.tc_err_d, w.tc_err_h, 0));
  return Status::ok();
}

Status nn_check(const WarmModel &w) {
  const int code = w.tc_err_h ? *(volatile int *)w.tc_err_h : 0;
  if (code) return Status{GOPS_ERR_CUDA, "warm start: a tensor-core GEMM handshake timed out (stage " +
                                             std::to_string(code) + ")"};
  return Status::ok();
}

Status nn_init_params(WarmModel &w) {
  std::vector<float> p(kPCount, 0.f);
  uint64_t ctr = w.cfg.seed ^ 0x5EEDF00Dull;
  auto uni = [&](float a) {  // uniform in [-a, a) from 24 random bits
    const uint64_t z = mix64(ctr++);
    return a * ((float)(z >> 40) * (1.0f / 8388608.0f) - 1.0f);
  };
  const float a1 = 1.0f / std::sqrt((float)(2 * kWFeat)), a2 = 1.0f / std::sqrt((float)(2 * kWH));
  for (int k = 0; k < 2 * kWFeat; ++k)
    for (int j = 0; j < kWH; ++j) p[kPW1 + k * kWH + j] = uni(a1);
  for (int k = 0; k < 2 * kWH; ++k)
    for (int j = 0; j < kWH; ++j) p[kPW2 + k * kWH + j] = uni(a2);
  // w3 = b3 = 0: the untrained network gives w = 1 (uniform within a cluster)
  GOPS_CUDA_TRY(cudaMemcpyAsync(w.params, p.data(), sizeof(float) * kPCount, cudaMemcpyHostToDevice, w.ctx->stream));
  GOPS_CUDA_TRY(cudaMemsetAsync(w.adam_m, 0, sizeof(float) * kPCount, w.ctx->stream));
  GOPS_CUDA_TRY(cudaMemsetAsync(w.adam_v, 0, sizeof(float) * kPCount, w.ctx->stream));
  GOPS_CUDA_TRY(cudaStreamSynchronize(w.ctx->stream));
  w.adam_t = 0;
  return nn_refresh_bf16(w);
}

Status nn_refresh_bf16(WarmModel &w) {
  refresh_bf16<<<(2 * kWH * kWH + 255) / 256, 256, 0, w.ctx->stream>>>(w.params, w.w1t, w.w2t, w.w2);
  GOPS_CUDA_TRY(cudaGetLastError());
  w.weights_fresh = false;
  return Status::ok();
}

Status nn_forward(WarmModel &w) {
  cudaStream_t s = w.ctx->stream;
  GOPS_TRY(launch_rows<kWIn>(w, w.x1, kWIn, nullptr, w.w1t, 1, w.h1, kWH));
  agg_in_128<<<blocks_for(w.n, 8, w.ctx->num_sms * 16), 256, 0, s>>>(w.in_rp, w.in_col, w.inv_in, w.h1, w.n, w.a1);
  GOPS_CUDA_TRY(cudaGetLastError());
  const TcEpi e2{w.h2, kWH, w.params + kPB2, w.params + kPW3, w.w};
  GOPS_TRY(tc_layer2(w.ctx, w.h1, w.a1, w.w2t, w.n, e2, w.tc_err_d));
  cluster_sums<<<blocks_for(w.r, 8, 1024), 256, 0, s>>>(w.members, w.cl_off, w.r, w.w, w.cw);
  GOPS_CUDA_TRY(cudaGetLastError());
  w.weights_fresh = true;
  return Status::ok();
}

Status nn_backward(WarmModel &w) {
  cudaStream_t s = w.ctx->stream;
  const int64_t heads = (w.n + kHeadRows - 1) / kHeadRows;
  head_backward<<<(unsigned)std::max<int64_t>(heads, 1), 256, 0, s>>>(w.du, w.h2, w.params + kPW3, w.n, w.g2, w.part);
  GOPS_CUDA_TRY(cudaGetLastError());
  // db2, dw3 and db3 are contiguous in the parameter layout
  static_assert(kPW3 == kPB2 + kWH && kPB3 == kPW3 + kWH, "head parameter layout");
  sum_parts<<<2, 256, 0, s>>>(w.part, std::max<int64_t>(heads, 1), 2 * kWH + 1, 2 * kWH + 1, w.grad + kPB2);
  GOPS_CUDA_TRY(cudaGetLastError());
  GOPS_TRY(launch_reduce<2 * kWH>(w, w.h1, kWH, w.a1, w.g2, w.grad + kPW2));
  const TcEpi e{w.gx, 2 * kWH, nullptr, nullptr, nullptr};
  GOPS_TRY(tc_input_grad(w.ctx, w.g2, w.w2, w.n, e, w.tc_err_d));
  h1_backward<<<blocks_for(w.n, 8, w.ctx->num_sms * 16), 256, 0, s>>>(w.out_rp, w.out_col, w.inv_in, w.gx, w.h1,
                                                                       w.n, w.g2);
  GOPS_CUDA_TRY(cudaGetLastError());
  GOPS_TRY(launch_reduce<kWIn>(w, w.x1, kWIn, nullptr, w.g2, w.grad + kPW1));
  return Status::ok();
}

Status nn_adam(WarmModel &w, float lr) {
  ++w.adam_t;
  const float c1 = 1.0f - (float)std::pow(0.9, (double)w.adam_t);
  const float c2 = 1.0f - (float)std::pow(0.999, (double)w.adam_t);
  adam_step<<<(kPCount + 255) / 256, 256, 0, w.ctx->stream>>>(w.params, w.grad, w.adam_m, w.adam_v, kPCount, lr, c1,
                                                              c2);
  GOPS_CUDA_TRY(cudaGetLastError());
  return nn_refresh_bf16(w);
}

}  // namespace gops
