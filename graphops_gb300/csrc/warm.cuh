// The learned warm start behind gops_warm_* (include/gops.h): model state and
// the kernels shared by warm.cu (graph-side state, push, least squares,
// drivers) and warm_nn.cu (the message-passing network: BF16 tensor-core
// GEMMs with FP32 accumulation, forward, backward, Adam).
#pragma once
#include <cuda_bf16.h>

#include "objects.cuh"

namespace gops {

constexpr int kWH = 128;          // MPNN hidden width
constexpr int kWCode = 16;        // random-projection code width
constexpr int kWFeat = 18;        // node features: log1p(out-deg), log1p(in-deg), code
constexpr int kWIn = 48;          // layer-1 input [x, mean_in x, 1, 0 ...] (36 used + bias column)
constexpr int kWBiasCol = 2 * kWFeat;  // column of the constant 1 (layer-1 bias row of W1)
constexpr int kWY = 2 * kWCode;   // clustering space: [code, mean_in code]
constexpr int kWMaxClusters = 256;
constexpr int kWMaxBatch = 32;    // sets per loss evaluation / Adam step
constexpr double kWFix = 1099511627776.0;  // 2^40: fixed-point scale of push sums

// parameter layout (FP32 master copy, one array)
constexpr int kPW1 = 0;                       // W1 [kWIn][kWH]
constexpr int kPW2 = kPW1 + kWIn * kWH;       // W2 [2*kWH][kWH]
constexpr int kPB2 = kPW2 + 2 * kWH * kWH;    // b2 [kWH]
constexpr int kPW3 = kPB2 + kWH;              // w3 [kWH]
constexpr int kPB3 = kPW3 + kWH;              // b3 [1]
constexpr int kPCount = kPB3 + 1;

struct WarmModel {
  Ctx *ctx = nullptr;  // the creating context (not dereferenced on destroy)
  int device = 0;
  const Graph *graph = nullptr;
  gops_warm_config cfg{};
  int64_t n = 0, m = 0;
  int r = 0;  // clusters
  // original-order CSRs
  int64_t *out_rp = nullptr;
  int32_t *out_col = nullptr;
  int64_t *in_rp = nullptr;
  int32_t *in_col = nullptr;
  float *inv_out = nullptr;  // 1/out-degree (0 when dangling)
  float *inv_in = nullptr;   // 1/in-degree (0 when none)
  // graph-side features
  float *code = nullptr;           // n x kWCode
  __nv_bfloat16 *x1 = nullptr;     // n x kWIn
  int32_t *cluster = nullptr;      // n
  int32_t *members = nullptr;      // n, nodes sorted by (cluster, id)
  int32_t *cl_off = nullptr;       // r + 1
  // parameters
  float *params = nullptr;         // kPCount (FP32 master)
  float *adam_m = nullptr, *adam_v = nullptr;
  __nv_bfloat16 *w1t = nullptr;    // W1^T  [kWH][kWIn]
  __nv_bfloat16 *w2t = nullptr;    // W2^T  [kWH][2*kWH]
  __nv_bfloat16 *w2 = nullptr;     // W2    [2*kWH][kWH]
  long long adam_t = 0;
  float *coupling = nullptr;       // K [(2r+1) x r]
  bool coupling_set = false;
  // activations (n rows)
  __nv_bfloat16 *h1 = nullptr, *a1 = nullptr, *h2 = nullptr;  // n x kWH each
  __nv_bfloat16 *g2 = nullptr, *gx = nullptr;                 // backward: dH2, [dH1 | dAgg] n x 2kWH
  float *w = nullptr;              // n: exp(u)
  float *du = nullptr;             // n: dL/du
  float *cw = nullptr;             // r: sum of w per cluster
  float *grad = nullptr;           // kPCount
  int *tc_err_h = nullptr;         // pinned, mapped: set by a tensor-core GEMM whose handshake wait ran out
  int *tc_err_d = nullptr;         // the same flag, device address
  float *part = nullptr;           // GEMM / reduction partials
  int64_t part_cap = 0;
  bool weights_fresh = false;      // w/cw computed for the current parameters
  // push scratch: fixed-point local terms, set-major, `push_cap` sets
  long long *push = nullptr;
  int64_t push_cap = 0;
  double *mix = nullptr;           // sets x (2r+1)
  double *tmass = nullptr;         // sets
  double *r1c = nullptr;           // sets
  int32_t *over = nullptr;         // sets: push budget exceeded
  float *coef = nullptr;           // sets x r
  int64_t set_cap = 0;
  int64_t *d_sptr = nullptr;       // seed sets of the current call
  int32_t *d_sidx = nullptr;
  int64_t sidx_cap = 0, sptr_cap = 0;
  // cluster distributions of the 3- and 4-step walks from each node:
  // t3[u][c] = (H^T P^3 e_u)[c], t4[u][c] = (H^T P^4 e_u)[c]  (n x r each)
  float *t3 = nullptr, *t4 = nullptr;
  // training
  float *targets = nullptr;        // targets_cap x n: PPR vectors, then their tails
  int64_t targets_cap = 0;
  int8_t *gsign = nullptr;         // kWMaxBatch x n: sign of the loss residual
  float *csum = nullptr;           // kWMaxBatch x r: sum of sign * w per cluster
  double *ymass = nullptr;         // push_cap x r: cluster masses of the target tails
  double *gram = nullptr;          // (2r+1)^2: least-squares normal matrix
  double *rhs = nullptr;           // (2r+1) x r
  double *chol = nullptr;          // (2r+1)^2 scratch
  double *lpart = nullptr;         // loss partials
  int64_t gram_sets = 0;           // targets accumulated into gram/rhs
  // learned batch
  float *x0 = nullptr;
  int64_t x0_cap = 0;              // sets
  ~WarmModel();
};

// warm_nn.cu
Status nn_alloc(WarmModel &w);
Status nn_init_params(WarmModel &w);
Status nn_refresh_bf16(WarmModel &w);
// w = exp(MPNN(x1)) and cw; keeps the activations for nn_backward
Status nn_forward(WarmModel &w);
// gradient of the parameters from du (dL/du), into w.grad
Status nn_backward(WarmModel &w);
Status nn_adam(WarmModel &w, float lr);
// error when a tensor-core GEMM of the network reported a failed handshake
// (read after a stream synchronisation)
Status nn_check(const WarmModel &w);

}  // namespace gops

struct gops_warm {
  gops::WarmModel impl;
};
