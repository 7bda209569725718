// tcgen05 / TMA row-tile GEMMs of the warm start's network (warm_tc.cu).
#pragma once
#include <cuda_bf16.h>

#include "objects.cuh"

namespace gops {

enum { kTcRelu = 0, kTcLayer2 = 1, kTcStore = 2 };

struct TcEpi {
  __nv_bfloat16 *out;  // M x ld
  int ld;
  const float *bias;   // layer 2: b2
  const float *head;   // layer 2: w3 (128) then b3
  float *w;            // layer 2: exp(u) per row
};

// H2 = relu([h1 | a1] w2t^T + b2) (n x 128, e.out), w = exp(H2 w3 + b3).
// h1, a1: n x 128; w2t: W2^T [128][256].  err: device flag set (nonzero) when
// a handshake wait ran out.
Status tc_layer2(Ctx *ctx, const __nv_bfloat16 *h1, const __nv_bfloat16 *a1, const __nv_bfloat16 *w2t, int64_t n,
                 const TcEpi &e, int *err);
// [dH1 | dA1] = g2 W2^T (n x 256, e.out): g2 n x 128, w2 = W2 [256][128].
Status tc_input_grad(Ctx *ctx, const __nv_bfloat16 *g2, const __nv_bfloat16 *w2, int64_t n, const TcEpi &e,
                     int *err);

}  // namespace gops
