// Katz centrality (src/katz.rs:136-201) and eigenvector centrality
// (src/eigenvector.rs:49-125): the same pull SpMV power iteration as
// PageRank, with the reference's update, L1 stopping rule (strict <) and
// diagnostics.  Both run in FP64: their tolerances are absolute while their
// scores are not normalised to sum 1 (Katz grows with beta and the walk
// counts), so FP32 cannot reproduce the reference's iteration counts.  The
// per-edge work is one FP64 add, far below the GPU's FP64 rate at these
// gather-bound speeds.  Every sum is taken in a fixed order (per sub-warp, per
// block, then over blocks), so results are bit-reproducible.
#include <cmath>
#include <cstdio>
#include <utility>
#include <vector>

#include "objects.cuh"

namespace gops {
namespace {

constexpr int kCThreads = 256;
constexpr int kSub = 8;  // lanes per row
constexpr int kCBlocks = 1024;

// sum over the kSub lanes of this lane's group.  The mask names the group
// only: the groups of a warp run different numbers of rows (a group past the
// last row runs none), so a full-warp mask would name lanes that never
// arrive at the shuffle.
__device__ __forceinline__ double sub_sum(double v) {
  const unsigned gmask = ((1u << kSub) - 1u) << ((threadIdx.x & 31) & ~(kSub - 1));
#pragma unroll
  for (int o = kSub / 2; o > 0; o >>= 1) v += __shfl_xor_sync(gmask, v, o, kSub);
  return v;
}

// block-level fixed-order sum of one value per thread into part[blockIdx.x * stride + slot]
__device__ __forceinline__ void block_part(double v, double *sh, double *part, int stride, int slot) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(int64_t)blockIdx.x * stride + slot] = sh[0];
  __syncthreads();
}

// Katz step over the relabelled, padded in-edge CSR (x has n + 1 entries,
// x[n] = 0 for the padding edges): y[v] = beta + alpha * sum_{u -> v} x[u]
// (src/katz.rs:166-173); part[b] = this block's sum of |x - y|.
__global__ void __launch_bounds__(kCThreads) katz_step(const int64_t *__restrict__ rp, const int32_t *__restrict__ col,
                                                       int64_t n, double alpha, double beta,
                                                       const double *__restrict__ x, double *__restrict__ y,
                                                       double *__restrict__ part) {
  __shared__ double sh[kCThreads];
  const int lane = threadIdx.x & (kSub - 1);
  const int64_t groups = (int64_t)gridDim.x * (kCThreads / kSub);
  double dl = 0.0;
  for (int64_t v = (int64_t)blockIdx.x * (kCThreads / kSub) + threadIdx.x / kSub; v < n; v += groups) {
    double s = 0.0;
    for (int64_t e = rp[v] + lane; e < rp[v + 1]; e += kSub) s += x[col[e]];
    s = sub_sum(s);
    const double yv = beta + alpha * s;
    if (lane == 0) {
      y[v] = yv;
      dl += fabs(x[v] - yv);
    }
  }
  block_part(dl, sh, part, 1, 0);
}

// Eigenvector step over the out-adjacency (original ids): y[v] = x[v] +
// sum_{u in neighbors(v)} x[u] (src/eigenvector.rs:72-81); part[b] = (sum y^2, sum y).
__global__ void __launch_bounds__(kCThreads) eig_step(const int64_t *__restrict__ rp, const int32_t *__restrict__ col,
                                                      int64_t n, const double *__restrict__ x, double *__restrict__ y,
                                                      double *__restrict__ part) {
  __shared__ double sh[kCThreads];
  const int lane = threadIdx.x & (kSub - 1);
  const int64_t groups = (int64_t)gridDim.x * (kCThreads / kSub);
  double sq = 0.0, su = 0.0;
  for (int64_t v = (int64_t)blockIdx.x * (kCThreads / kSub) + threadIdx.x / kSub; v < n; v += groups) {
    double s = 0.0;
    for (int64_t e = rp[v] + lane; e < rp[v + 1]; e += kSub) s += x[col[e]];
    s = sub_sum(s);
    const double yv = x[v] + s;
    if (lane == 0) {
      y[v] = yv;
      sq += yv * yv;
      su += yv;
    }
  }
  block_part(sq, sh, part, 2, 0);
  block_part(su, sh, part, 2, 1);
}

// out[j] = sum over blocks of part[b * stride + j] (one block, fixed order)
__global__ void sum_blocks(const double *__restrict__ part, int nb, int stride, double *__restrict__ out) {
  __shared__ double sh[kCThreads];
  for (int j = 0; j < stride; ++j) {
    double t = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) t += part[(int64_t)b * stride + j];
    sh[threadIdx.x] = t;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[j] = sh[0];
    __syncthreads();
  }
}

// L2 normalisation with the positive-sum sign (src/eigenvector.rs:84-95),
// then part[b] = this block's sum of |x - y| (src/eigenvector.rs:98-102)
__global__ void __launch_bounds__(kCThreads) eig_scale(int64_t n, const double *__restrict__ sums,
                                                       const double *__restrict__ x, double *__restrict__ y,
                                                       double *__restrict__ part) {
  __shared__ double sh[kCThreads];
  const double norm = sqrt(sums[0]);
  const double sign = sums[1] >= 0.0 ? 1.0 : -1.0;
  double dl = 0.0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    double yv = y[v];
    if (norm > 0.0) {
      yv = yv * sign / norm;
      y[v] = yv;
    }
    dl += fabs(x[v] - yv);
  }
  block_part(dl, sh, part, 1, 0);
}

// HITS: y[v] = sum over the row's edges of x[col] (no self term); part[b] =
// this block's sum of y^2.  Rows of the relabelled in-CSR (x has n+1 entries,
// x[n] = 0) or of the out-adjacency.
__global__ void __launch_bounds__(kCThreads) pull_sum(const int64_t *__restrict__ rp, const int32_t *__restrict__ col,
                                                      int64_t n, const double *__restrict__ x, double *__restrict__ y,
                                                      double *__restrict__ part) {
  __shared__ double sh[kCThreads];
  const int lane = threadIdx.x & (kSub - 1);
  const int64_t groups = (int64_t)gridDim.x * (kCThreads / kSub);
  double sq = 0.0;
  for (int64_t v = (int64_t)blockIdx.x * (kCThreads / kSub) + threadIdx.x / kSub; v < n; v += groups) {
    double s = 0.0;
    for (int64_t e = rp[v] + lane; e < rp[v + 1]; e += kSub) s += x[col[e]];
    s = sub_sum(s);
    if (lane == 0) {
      y[v] = s;
      sq += s * s;
    }
  }
  block_part(sq, sh, part, 1, 0);
}

// HITS l2_normalize (src/centrality.rs:168-175) of y in place (skipped when
// the norm is 0), then part[b] = this block's sum of (x - y)^2 for l2_diff
// (src/centrality.rs:177-183); xo indexes x in y's order through `map`
// (map == nullptr: same order)
__global__ void __launch_bounds__(kCThreads) l2_scale(int64_t n, const double *__restrict__ sums,
                                                      const double *__restrict__ x, const int32_t *__restrict__ map,
                                                      double *__restrict__ y, double *__restrict__ part) {
  __shared__ double sh[kCThreads];
  const double norm = sqrt(sums[0]);
  double dl = 0.0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    double yv = y[v];
    if (norm > 0.0) {
      yv = yv / norm;
      y[v] = yv;
    }
    const double t = x[map ? map[v] : v] - yv;
    dl += t * t;
  }
  block_part(dl, sh, part, 1, 0);
}

// out[i] = x[perm[i]] (original order -> relabelled order); out[n] = 0
__global__ void permute_to_rows(const double *x, const int32_t *perm, int64_t n, double *out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = i < n ? x[perm[i]] : 0.0;
}

__global__ void fill_f64(double *a, int64_t n, double v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) a[i] = v;
}

__global__ void unpermute_f64(const double *x, const int32_t *perm, int64_t n, double *out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[perm[i]] = x[i];
}

struct Bufs {
  double *x = nullptr, *y = nullptr, *part = nullptr, *sums = nullptr, *out = nullptr;
  ~Bufs() {
    cudaFree(x); cudaFree(y); cudaFree(part); cudaFree(sums); cudaFree(out);
  }
};

int grid_rows(int64_t n) {
  return blocks_for(n, kCThreads / kSub, kCBlocks);
}

}  // namespace

Status katz_run(Ctx *ctx, const Graph *g, const gops_katz_config *cfg, double *scores, gops_run *run) {
  ctx->stats = gops_stats{};
  const int64_t n = g->n;
  *run = gops_run{0, 0.0, 1, 0};
  if (n == 0) return Status::ok();  // src/katz.rs:138-145
  cudaStream_t s = ctx->stream;
  Bufs b;
  const int nb = grid_rows(n);
  GOPS_CUDA_TRY(cudaMalloc(&b.x, sizeof(double) * (n + 1)));
  GOPS_CUDA_TRY(cudaMalloc(&b.y, sizeof(double) * (n + 1)));
  GOPS_CUDA_TRY(cudaMalloc(&b.part, sizeof(double) * nb));
  GOPS_CUDA_TRY(cudaMalloc(&b.sums, sizeof(double) * 2));
  GOPS_CUDA_TRY(cudaMalloc(&b.out, sizeof(double) * n));
  fill_f64<<<blocks_for(n, 256, 4096), 256, 0, s>>>(b.x, n, cfg->beta);  // src/katz.rs:149
  GOPS_CUDA_TRY(cudaMemsetAsync(b.x + n, 0, sizeof(double), s));
  GOPS_CUDA_TRY(cudaMemsetAsync(b.y + n, 0, sizeof(double), s));
  uint64_t it = 0, launches = 1;
  double last = INFINITY;  // src/katz.rs:158
  bool conv = false;
  GOPS_CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  for (uint64_t k = 0; k < cfg->max_iterations; ++k) {
    ++it;
    katz_step<<<nb, kCThreads, 0, s>>>(g->in_rp, g->in_col, n, cfg->alpha, cfg->beta, b.x, b.y, b.part);
    sum_blocks<<<1, kCThreads, 0, s>>>(b.part, nb, 1, b.sums);
    launches += 2;
    double d = 0.0;
    GOPS_CUDA_TRY(cudaMemcpyAsync(&d, b.sums, sizeof(double), cudaMemcpyDeviceToHost, s));
    GOPS_CUDA_TRY(cudaStreamSynchronize(s));
    last = d;
    std::swap(b.x, b.y);
    if (d < cfg->tolerance) {
      conv = true;
      break;
    }
  }
  unpermute_f64<<<blocks_for(n, 256, 4096), 256, 0, s>>>(b.x, g->perm, n, b.out);
  GOPS_CUDA_TRY(cudaGetLastError());
  GOPS_CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
  if (scores) {
    GOPS_CUDA_TRY(cudaMemcpyAsync(scores, b.out, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    ctx->stats.d2h_bytes += sizeof(double) * n;
  }
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
  ctx->stats.solve_ms = ms;
  ctx->stats.kernel_launches = launches + 1;
  ctx->stats.iterations = it;
  *run = gops_run{it, last, conv ? 1 : 0, 0};
  return Status::ok();
}

Status eigenvector_run(Ctx *ctx, const Graph *g, uint64_t max_iterations, double tolerance, double *scores,
                       gops_run *run) {
  ctx->stats = gops_stats{};
  const int64_t n = g->n;
  *run = gops_run{0, 0.0, 1, 0};
  if (n == 0) return Status::ok();  // src/eigenvector.rs:55-62
  if (!g->out_rp) return Status{GOPS_ERR_INTERNAL, "graph has no out-adjacency"};
  cudaStream_t s = ctx->stream;
  Bufs b;
  const int nb = grid_rows(n);
  const int nbs = blocks_for(n, 256, kCBlocks);
  GOPS_CUDA_TRY(cudaMalloc(&b.x, sizeof(double) * n));
  GOPS_CUDA_TRY(cudaMalloc(&b.y, sizeof(double) * n));
  GOPS_CUDA_TRY(cudaMalloc(&b.part, sizeof(double) * 2 * std::max(nb, nbs)));
  GOPS_CUDA_TRY(cudaMalloc(&b.sums, sizeof(double) * 2));
  fill_f64<<<blocks_for(n, 256, 4096), 256, 0, s>>>(b.x, n, 1.0 / std::sqrt((double)n));  // src/eigenvector.rs:65
  uint64_t it = 0, launches = 1;
  double last = 0.0;  // src/eigenvector.rs:68
  bool conv = false;
  GOPS_CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  for (uint64_t k = 0; k < max_iterations; ++k) {
    it = k + 1;
    eig_step<<<nb, kCThreads, 0, s>>>(g->out_rp, g->out_col, n, b.x, b.y, b.part);
    sum_blocks<<<1, kCThreads, 0, s>>>(b.part, nb, 2, b.sums);
    eig_scale<<<nbs, kCThreads, 0, s>>>(n, b.sums, b.x, b.y, b.part);
    sum_blocks<<<1, kCThreads, 0, s>>>(b.part, nbs, 1, b.sums);
    launches += 4;
    double d = 0.0;
    GOPS_CUDA_TRY(cudaMemcpyAsync(&d, b.sums, sizeof(double), cudaMemcpyDeviceToHost, s));
    GOPS_CUDA_TRY(cudaStreamSynchronize(s));
    last = d;
    std::swap(b.x, b.y);
    if (d < tolerance) {
      conv = true;
      break;
    }
  }
  GOPS_CUDA_TRY(cudaGetLastError());
  GOPS_CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
  if (scores) {
    GOPS_CUDA_TRY(cudaMemcpyAsync(scores, b.x, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    ctx->stats.d2h_bytes += sizeof(double) * n;
  }
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
  ctx->stats.solve_ms = ms;
  ctx->stats.kernel_launches = launches;
  ctx->stats.iterations = it;
  *run = gops_run{it, last, conv ? 1 : 0, 0};
  return Status::ok();
}

// hits (src/centrality.rs:114-166): hub = auth = 1/sqrt(n); each step
// auth' = l2n(A^T hub), hub' = l2n(A auth'); stop when both L2 changes < tol.
// The reference returns (hub, auth) only; `run` adds the step count, the
// larger of the two L2 changes, and whether both fell below tol.
Status hits_run(Ctx *ctx, const Graph *g, uint64_t max_iterations, double tolerance, double *hub_out,
                double *auth_out, gops_run *run) {
  ctx->stats = gops_stats{};
  const int64_t n = g->n;
  *run = gops_run{0, 0.0, 0, 0};
  if (n == 0) {
    run->converged = 1;
    return Status::ok();
  }
  if (!g->out_rp) return Status{GOPS_ERR_INTERNAL, "graph has no out-adjacency"};
  cudaStream_t s = ctx->stream;
  struct H {
    double *hub = nullptr, *auth = nullptr, *nhub = nullptr, *nauth_r = nullptr, *nauth = nullptr,
           *hub_r = nullptr, *part = nullptr, *sums = nullptr;
    ~H() {
      cudaFree(hub); cudaFree(auth); cudaFree(nhub); cudaFree(nauth_r); cudaFree(nauth); cudaFree(hub_r);
      cudaFree(part); cudaFree(sums);
    }
  } h;
  const int nb = grid_rows(n), nbs = blocks_for(n, 256, kCBlocks);
  GOPS_CUDA_TRY(cudaMalloc(&h.hub, sizeof(double) * n));
  GOPS_CUDA_TRY(cudaMalloc(&h.auth, sizeof(double) * n));
  GOPS_CUDA_TRY(cudaMalloc(&h.nhub, sizeof(double) * n));
  GOPS_CUDA_TRY(cudaMalloc(&h.nauth_r, sizeof(double) * n));
  GOPS_CUDA_TRY(cudaMalloc(&h.nauth, sizeof(double) * n));
  GOPS_CUDA_TRY(cudaMalloc(&h.hub_r, sizeof(double) * (n + 1)));
  GOPS_CUDA_TRY(cudaMalloc(&h.part, sizeof(double) * std::max(nb, nbs)));
  GOPS_CUDA_TRY(cudaMalloc(&h.sums, sizeof(double) * 4));
  const double init = 1.0 / std::sqrt((double)n);  // src/centrality.rs:130
  fill_f64<<<blocks_for(n, 256, 4096), 256, 0, s>>>(h.hub, n, init);
  fill_f64<<<blocks_for(n, 256, 4096), 256, 0, s>>>(h.auth, n, init);
  uint64_t it = 0, launches = 2;
  double last = 0.0;
  bool conv = false;
  GOPS_CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  for (uint64_t k = 0; k < max_iterations; ++k) {
    it = k + 1;
    // authority: pull over the in-edge rows (relabelled), back to original order
    permute_to_rows<<<blocks_for(n + 1, 256, 4096), 256, 0, s>>>(h.hub, g->perm, n, h.hub_r);
    pull_sum<<<nb, kCThreads, 0, s>>>(g->in_rp, g->in_col, n, h.hub_r, h.nauth_r, h.part);
    sum_blocks<<<1, kCThreads, 0, s>>>(h.part, nb, 1, h.sums);
    l2_scale<<<nbs, kCThreads, 0, s>>>(n, h.sums, h.auth, g->perm, h.nauth_r, h.part);
    sum_blocks<<<1, kCThreads, 0, s>>>(h.part, nbs, 1, h.sums + 2);
    unpermute_f64<<<blocks_for(n, 256, 4096), 256, 0, s>>>(h.nauth_r, g->perm, n, h.nauth);
    // hub: pull over the out-adjacency (original order)
    pull_sum<<<nb, kCThreads, 0, s>>>(g->out_rp, g->out_col, n, h.nauth, h.nhub, h.part);
    sum_blocks<<<1, kCThreads, 0, s>>>(h.part, nb, 1, h.sums);
    l2_scale<<<nbs, kCThreads, 0, s>>>(n, h.sums, h.hub, nullptr, h.nhub, h.part);
    sum_blocks<<<1, kCThreads, 0, s>>>(h.part, nbs, 1, h.sums + 3);
    launches += 10;
    double d[2] = {0.0, 0.0};
    GOPS_CUDA_TRY(cudaMemcpyAsync(d, h.sums + 2, sizeof(double) * 2, cudaMemcpyDeviceToHost, s));
    GOPS_CUDA_TRY(cudaStreamSynchronize(s));
    const double ad = std::sqrt(d[0]), hd = std::sqrt(d[1]);
    last = std::max(ad, hd);
    std::swap(h.auth, h.nauth);
    std::swap(h.hub, h.nhub);
    if (ad < tolerance && hd < tolerance) {
      conv = true;
      break;
    }
  }
  GOPS_CUDA_TRY(cudaGetLastError());
  GOPS_CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
  if (hub_out) GOPS_CUDA_TRY(cudaMemcpyAsync(hub_out, h.hub, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  if (auth_out) GOPS_CUDA_TRY(cudaMemcpyAsync(auth_out, h.auth, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
  ctx->stats.solve_ms = ms;
  ctx->stats.kernel_launches = launches;
  ctx->stats.iterations = it;
  ctx->stats.d2h_bytes = sizeof(double) * n * ((hub_out ? 1 : 0) + (auth_out ? 1 : 0));
  *run = gops_run{it, last, conv ? 1 : 0, 0};
  return Status::ok();
}

}  // namespace gops

using namespace gops;

extern "C" {

int gops_katz_config_validate(const gops_katz_config *cfg, char *msg, size_t msg_cap) {
  auto fail = [&](const char *t) {
    if (msg && msg_cap) std::snprintf(msg, msg_cap, "%s", t);
    return GOPS_ERR_INVALID;
  };
  if (!cfg) return fail("null config");
  // src/katz.rs:60-86, same order and messages
  if (!std::isfinite(cfg->alpha) || cfg->alpha <= 0.0) return fail("alpha must be finite and > 0");
  if (cfg->alpha >= 1.0)
    return fail("alpha must be < 1 (required for convergence; tighter bound alpha < 1/spectral_radius(A) "
                "may be needed for large graphs)");
  if (!std::isfinite(cfg->beta)) return fail("beta must be finite");
  if (cfg->max_iterations == 0) return fail("max_iterations must be > 0");
  if (!std::isfinite(cfg->tolerance) || cfg->tolerance <= 0.0) return fail("tolerance must be finite and > 0");
  return GOPS_OK;
}

int gops_katz_run(gops_ctx *ctx, const gops_graph *g, const gops_katz_config *cfg, double *scores, gops_run *run) {
  if (!ctx) return GOPS_ERR_INVALID;
  Ctx &c = ctx->impl;
  if (!g || !cfg || !run) return c.set(Status{GOPS_ERR_INVALID, "null argument"});
  if (g->impl.ctx != &c) return c.set(Status{GOPS_ERR_INVALID, "graph belongs to another context"});
  cudaSetDevice(c.device);
  return c.set(katz_run(&c, &g->impl, cfg, scores, run));
}

int gops_eigenvector_run(gops_ctx *ctx, const gops_graph *g, uint64_t max_iterations, double tolerance,
                         double *scores, gops_run *run) {
  if (!ctx) return GOPS_ERR_INVALID;
  Ctx &c = ctx->impl;
  if (!g || !run) return c.set(Status{GOPS_ERR_INVALID, "null argument"});
  if (g->impl.ctx != &c) return c.set(Status{GOPS_ERR_INVALID, "graph belongs to another context"});
  cudaSetDevice(c.device);
  return c.set(eigenvector_run(&c, &g->impl, max_iterations, tolerance, scores, run));
}

int gops_hits_run(gops_ctx *ctx, const gops_graph *g, uint64_t max_iterations, double tolerance, double *hub,
                  double *auth, gops_run *run) {
  if (!ctx) return GOPS_ERR_INVALID;
  Ctx &c = ctx->impl;
  if (!g || !run) return c.set(Status{GOPS_ERR_INVALID, "null argument"});
  if (g->impl.ctx != &c) return c.set(Status{GOPS_ERR_INVALID, "graph belongs to another context"});
  cudaSetDevice(c.device);
  return c.set(hits_run(&c, &g->impl, max_iterations, tolerance, hub, auth, run));
}

}  // extern "C"
