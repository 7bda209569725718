// Katz centrality (src/katz.rs:136-201) and eigenvector centrality
// (src/eigenvector.rs:49-125): the same pull SpMV power iteration as
// PageRank, with the reference's update, L1 stopping rule (strict <) and
// diagnostics.  Both run in FP64: their tolerances are absolute while their
// scores are not normalised to sum 1 (Katz grows with beta and the walk
// counts), so FP32 cannot reproduce the reference's iteration counts.  The
// per-edge work is one FP64 add, far below the GPU's FP64 rate at these
// gather-bound speeds.  Rows with at most kLong edges are summed by 8-lane
// groups; longer rows (power-law hubs, in- or out-degree) in kChunkE-edge
// chunks of a block each, whose sums are added in chunk order, so no hub row
// leaves a few lanes running long after the rest.  Every sum is taken in a
// fixed order (per sub-warp or chunk, per block, then over blocks), so
// results are bit-reproducible.
#include <cmath>
#include <cstdio>
#include <utility>
#include <vector>

#include "objects.cuh"
#include "primitives.cuh"

namespace gops {
namespace {

constexpr int kCThreads = 256;
constexpr int kSub = 8;  // lanes per row
constexpr int kCBlocks = 1024;
constexpr int64_t kLong = 2048;    // rows with more edges are summed in chunks, a block each
constexpr int64_t kLight = 8;      // rows with fewer edges are summed by one lane each
constexpr int64_t kChunkE = 8192;  // edges per chunk

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

// Per-row updates of the three pulls: y[v] from the row's own x[v] and its
// gathered sum s, and the contributions to the step's global sums.
struct KatzOp {  // y[v] = beta + alpha * sum_{u -> v} x[u] (src/katz.rs:166-173); sum |x - y|
  static constexpr int kSlots = 1;
  double alpha, beta;
  __device__ double y(double xv, double s) const { return beta + alpha * s; }
  __device__ void add(double xv, double yv, double (&acc)[2]) const { acc[0] += fabs(xv - yv); }
};
struct EigOp {  // y[v] = x[v] + sum_{u in neighbors(v)} x[u] (src/eigenvector.rs:72-81); sum y^2, sum y
  static constexpr int kSlots = 2;
  __device__ double y(double xv, double s) const { return xv + s; }
  __device__ void add(double, double yv, double (&acc)[2]) const {
    acc[0] += yv * yv;
    acc[1] += yv;
  }
};
struct SumOp {  // HITS: y[v] = sum over the row's edges (no self term); sum y^2
  static constexpr int kSlots = 1;
  __device__ double y(double, double s) const { return s; }
  __device__ void add(double, double yv, double (&acc)[2]) const { acc[0] += yv * yv; }
};

// Rows with at most kLong edges: kSub lanes per row, four gathers in flight
// per lane (each lane adds its edges e, e + kSub, ... in order).  Longer rows
// are skipped here and summed in chunks (chunk_sums / long_rows).  The four
// row groups of a warp run together until the longest of their rows ends, so
// rows are taken in non-increasing degree class: the in-edge CSR's rows
// already are (relabelled by in-degree); the out-adjacency, in the caller's
// node order, goes through a row order sorted by degree class.  x has
// n + 1 entries when the rows are the padded in-edge CSR (x[n] = 0 for the
// padding edges).  part[b * kSlots + j]: this block's global sums.
// Rows are taken in the order `order` lists them (n_rows of them) or, with
// order == nullptr, as 0..n_rows-1; the first n_heavy (the rows with at least
// kLight edges, long ones included, which are skipped) by kSub-lane groups,
// the rest (fewer than kLight edges: most rows of a power-law graph) by one
// lane each, which adds the row's edges in order.
template <class Op>
__global__ void __launch_bounds__(kCThreads) short_rows(const int64_t *__restrict__ rp, const int32_t *__restrict__ col,
                                                        const int32_t *__restrict__ order, int64_t n_heavy,
                                                        int64_t n_rows, Op op, const double *__restrict__ x,
                                                        double *__restrict__ y, double *__restrict__ part) {
  __shared__ double sh[kCThreads];
  const int lane = threadIdx.x & (kSub - 1);
  const int64_t groups = (int64_t)gridDim.x * (kCThreads / kSub);
  double acc[2] = {0.0, 0.0};
  for (int64_t i = (int64_t)blockIdx.x * (kCThreads / kSub) + threadIdx.x / kSub; i < n_heavy; i += groups) {
    const int64_t v = order ? (int64_t)order[i] : i;
    const int64_t eb = rp[v], ee = rp[v + 1];
    if (ee - eb > kLong) continue;  // a long row: chunk_sums / long_rows
    double s = 0.0;
    int64_t e = eb + lane;
    for (; e + 3 * kSub < ee; e += 4 * kSub) {
      const int32_t c0 = col[e], c1 = col[e + kSub], c2 = col[e + 2 * kSub], c3 = col[e + 3 * kSub];
      const double g0 = x[c0], g1 = x[c1], g2 = x[c2], g3 = x[c3];
      s += g0;
      s += g1;
      s += g2;
      s += g3;
    }
    for (; e < ee; e += kSub) s += x[col[e]];
    s = sub_sum(s);
    if (lane == 0) {
      const double yv = op.y(x[v], s);
      y[v] = yv;
      op.add(x[v], yv, acc);
    }
  }
  for (int64_t i = n_heavy + (int64_t)blockIdx.x * kCThreads + threadIdx.x; i < n_rows;
       i += (int64_t)gridDim.x * kCThreads) {
    const int64_t v = order ? (int64_t)order[i] : i;
    const int64_t eb = rp[v], ee = rp[v + 1];
    double s = 0.0;
    int64_t e = eb;
    for (; e + 4 <= ee; e += 4) {
      const int32_t c0 = col[e], c1 = col[e + 1], c2 = col[e + 2], c3 = col[e + 3];
      const double g0 = x[c0], g1 = x[c1], g2 = x[c2], g3 = x[c3];
      s += g0;
      s += g1;
      s += g2;
      s += g3;
    }
    for (; e < ee; ++e) s += x[col[e]];
    const double yv = op.y(x[v], s);
    y[v] = yv;
    op.add(x[v], yv, acc);
  }
  for (int j = 0; j < Op::kSlots; ++j) block_part(acc[j], sh, part, Op::kSlots, j);
}

// One block per chunk of kChunkE edges of a long row: cpart[t] = the sum of
// x over the chunk (per thread in edge order, then a fixed tree).
__global__ void __launch_bounds__(kCThreads) chunk_sums(const int64_t *__restrict__ rp, const int32_t *__restrict__ col,
                                                        const int32_t *__restrict__ rows,
                                                        const int64_t *__restrict__ first,
                                                        const int32_t *__restrict__ task_row,
                                                        const double *__restrict__ x, double *__restrict__ cpart) {
  __shared__ double sh[kCThreads];
  const int64_t t = blockIdx.x;
  const int32_t i = task_row[t];
  const int64_t v = rows[i];
  const int64_t eb = rp[v] + (t - first[i]) * kChunkE;
  const int64_t ee = min(rp[v + 1], eb + kChunkE);
  double s = 0.0;
  int64_t e = eb + threadIdx.x;
  for (; e + 3 * kCThreads < ee; e += 4 * kCThreads) {
    const int32_t c0 = col[e], c1 = col[e + kCThreads], c2 = col[e + 2 * kCThreads], c3 = col[e + 3 * kCThreads];
    const double g0 = x[c0], g1 = x[c1], g2 = x[c2], g3 = x[c3];
    s += g0;
    s += g1;
    s += g2;
    s += g3;
  }
  for (; e < ee; e += kCThreads) s += x[col[e]];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = kCThreads / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) cpart[t] = sh[0];
}

// Long rows, one thread each: the row's chunk sums added in chunk order,
// then the update; part[b * kSlots + j]: this block's global sums.
template <class Op>
__global__ void __launch_bounds__(kCThreads) long_rows(int64_t n_long, const int32_t *__restrict__ rows,
                                                       const int64_t *__restrict__ first,
                                                       const double *__restrict__ cpart, Op op,
                                                       const double *__restrict__ x, double *__restrict__ y,
                                                       double *__restrict__ part) {
  __shared__ double sh[kCThreads];
  double acc[2] = {0.0, 0.0};
  const int64_t i = (int64_t)blockIdx.x * kCThreads + threadIdx.x;
  if (i < n_long) {
    double s = 0.0;
    for (int64_t t = first[i]; t < first[i + 1]; ++t) s += cpart[t];
    const int64_t v = rows[i];
    const double yv = op.y(x[v], s);
    y[v] = yv;
    op.add(x[v], yv, acc);
  }
  for (int j = 0; j < Op::kSlots; ++j) block_part(acc[j], sh, part, Op::kSlots, j);
}

// ---- plan of the long rows of a CSR: the rows, their chunks
__global__ void long_flags(const int64_t *rp, int64_t n, int64_t *flag) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += (int64_t)gridDim.x * blockDim.x)
    flag[v] = v < n && rp[v + 1] - rp[v] > kLong ? 1 : 0;
}

__global__ void long_compact(const int64_t *rp, int64_t n, const int64_t *pos, int32_t *rows, int64_t *nch) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t d = rp[v + 1] - rp[v];
    if (d > kLong) {
      rows[pos[v]] = (int32_t)v;
      nch[pos[v]] = (d + kChunkE - 1) / kChunkE;
    }
  }
}

__global__ void long_tasks(const int64_t *first, int64_t n_long, int32_t *task_row) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_long; i += (int64_t)gridDim.x * blockDim.x)
    for (int64_t t = first[i]; t < first[i + 1]; ++t) task_row[t] = (int32_t)i;
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

// The long rows of a CSR (more than kLong edges) and their kChunkE-edge
// chunks, built once per call.
struct LongPlan {
  int64_t n_long = 0, n_chunks = 0;
  int32_t *rows = nullptr, *task_row = nullptr;
  int64_t *first = nullptr;
  double *cpart = nullptr;
  // rows of at most kLong edges by degree class, heaviest first (nullptr:
  // the rows are already in that order)
  int32_t *order = nullptr;
  int64_t n_short = 0;
  // leading rows (in the pull's order) with at least kLight edges
  int64_t n_heavy = 0;
  ~LongPlan() {
    cudaFree(rows); cudaFree(task_row); cudaFree(first); cudaFree(cpart); cudaFree(order);
  }
};

// key of row v for the row order: 12 - (degree class) for rows of at most
// kLong edges (class 0: no edge, c: 2^(c-1) <= degree < 2^c, so 0 for
// degree kLong), 15 for long rows, which sort last and are left out
__global__ void row_class_keys(const int64_t *rp, int64_t n, uint32_t *key) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t d = rp[v + 1] - rp[v];
    const int cls = d == 0 ? 0 : 64 - __clzll((unsigned long long)d);
    key[v] = d > kLong ? 15u : (uint32_t)(12 - cls);
  }
}

static_assert(kLong == 2048, "row_class_keys: degree classes 0..12 for rows of at most kLong edges");
static_assert(kLight == 8, "the light rows (degree < kLight) are the degree classes 0..3");

// *count += rows with lo <= degree <= hi
__global__ void count_rows(const int64_t *rp, int64_t n, int64_t lo, int64_t hi, unsigned long long *count) {
  unsigned long long c = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t d = rp[v + 1] - rp[v];
    c += d >= lo && d <= hi;
  }
  c = __reduce_add_sync(0xffffffffu, (unsigned)c);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

Status count_rows_host(cudaStream_t s, const int64_t *rp, int64_t n, int64_t lo, int64_t hi, int64_t *out) {
  unsigned long long *d = nullptr;
  GOPS_CUDA_TRY(cudaMalloc(&d, sizeof(unsigned long long)));
  struct Free {
    unsigned long long *p;
    ~Free() { cudaFree(p); }
  } fd{d};
  GOPS_CUDA_TRY(cudaMemsetAsync(d, 0, sizeof(unsigned long long), s));
  count_rows<<<blocks_for(n, 256, 4096), 256, 0, s>>>(rp, n, lo, hi, d);
  GOPS_CUDA_TRY(cudaGetLastError());
  unsigned long long h = 0;
  GOPS_CUDA_TRY(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s));
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  *out = (int64_t)h;
  return Status::ok();
}

// lp.order: the rows of at most kLong edges, stably sorted by degree class
// (heaviest first; one 4-bit radix pass)
Status build_row_order(cudaStream_t s, const int64_t *rp, int64_t n, LongPlan &lp) {
  uint32_t *buf = nullptr;
  GOPS_CUDA_TRY(cudaMalloc(&buf, sizeof(uint32_t) * 4 * n));
  struct Free {
    uint32_t *p;
    ~Free() { cudaFree(p); }
  } fb{buf};
  uint32_t *key_in = buf, *k = buf + n, *v = buf + 2 * n, *k2 = buf + 3 * n;
  GOPS_CUDA_TRY(cudaMalloc(&lp.order, sizeof(int32_t) * n));
  uint32_t *v2 = reinterpret_cast<uint32_t *>(lp.order);
  row_class_keys<<<blocks_for(n, 256, 4096), 256, 0, s>>>(rp, n, key_in);
  GOPS_CUDA_TRY(cudaGetLastError());
  bool alt = false;
  GOPS_TRY(radix_sort_index_u32(key_in, k, v, k2, v2, n, 4, &alt, s));
  if (!alt) GOPS_CUDA_TRY(cudaMemcpyAsync(lp.order, v, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));  // buf is freed on return
  lp.n_short = n - lp.n_long;
  return Status::ok();
}

Status build_long_plan_rows(cudaStream_t s, const int64_t *rp, int64_t n, LongPlan &lp) {
  int64_t *pos = nullptr;
  GOPS_CUDA_TRY(cudaMalloc(&pos, sizeof(int64_t) * (n + 1)));
  struct Free {
    int64_t *p;
    ~Free() { cudaFree(p); }
  } fp{pos};
  long_flags<<<blocks_for(n + 1, 256, 4096), 256, 0, s>>>(rp, n, pos);
  GOPS_CUDA_TRY(cudaGetLastError());
  GOPS_TRY(exclusive_scan_i64(pos, pos, n + 1, s));
  GOPS_CUDA_TRY(cudaMemcpyAsync(&lp.n_long, pos + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  if (lp.n_long == 0) return Status::ok();
  GOPS_CUDA_TRY(cudaMalloc(&lp.rows, sizeof(int32_t) * lp.n_long));
  GOPS_CUDA_TRY(cudaMalloc(&lp.first, sizeof(int64_t) * (lp.n_long + 1)));
  GOPS_CUDA_TRY(cudaMemsetAsync(lp.first + lp.n_long, 0, sizeof(int64_t), s));
  long_compact<<<blocks_for(n, 256, 4096), 256, 0, s>>>(rp, n, pos, lp.rows, lp.first);
  GOPS_CUDA_TRY(cudaGetLastError());
  GOPS_TRY(exclusive_scan_i64(lp.first, lp.first, lp.n_long + 1, s));
  GOPS_CUDA_TRY(cudaMemcpyAsync(&lp.n_chunks, lp.first + lp.n_long, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  GOPS_CUDA_TRY(cudaMalloc(&lp.task_row, sizeof(int32_t) * lp.n_chunks));
  GOPS_CUDA_TRY(cudaMalloc(&lp.cpart, sizeof(double) * lp.n_chunks));
  long_tasks<<<blocks_for(lp.n_long, 256, 4096), 256, 0, s>>>(lp.first, lp.n_long, lp.task_row);
  GOPS_CUDA_TRY(cudaGetLastError());
  return Status::ok();
}

// The long-row plan of a CSR, and with `ordered` the row order of its other rows.
// The in-edge CSR's rows are in non-increasing degree (long rows first, which
// the heavy loop skips); the ordered rows leave the long ones out.
Status build_long_plan(cudaStream_t s, const int64_t *rp, int64_t n, LongPlan &lp, bool ordered) {
  GOPS_TRY(build_long_plan_rows(s, rp, n, lp));
  if (ordered) GOPS_TRY(build_row_order(s, rp, n, lp));
  return count_rows_host(s, rp, n, kLight, ordered ? kLong : INT64_MAX, &lp.n_heavy);
}

// Blocks of part[] one pull writes: the short-row blocks, then the long-row blocks.
int pull_blocks(int64_t n, const LongPlan &lp) {
  return grid_rows(n) + (lp.n_long ? (int)ceil_div<int64_t>(lp.n_long, kCThreads) : 0);
}

// y = the pull of x over the rows of (rp, col) with the update op; part gets
// pull_blocks(n, lp) blocks of Op::kSlots sums.  Returns the launches.
template <class Op>
int pull(cudaStream_t s, const int64_t *rp, const int32_t *col, int64_t n, const LongPlan &lp, Op op,
         const double *x, double *y, double *part) {
  const int nb = grid_rows(n);
  short_rows<Op><<<nb, kCThreads, 0, s>>>(rp, col, lp.order, lp.n_heavy, lp.order ? lp.n_short : n, op, x, y, part);
  if (lp.n_long == 0) return 1;
  chunk_sums<<<(unsigned)lp.n_chunks, kCThreads, 0, s>>>(rp, col, lp.rows, lp.first, lp.task_row, x, lp.cpart);
  long_rows<Op><<<(unsigned)ceil_div<int64_t>(lp.n_long, kCThreads), kCThreads, 0, s>>>(
      lp.n_long, lp.rows, lp.first, lp.cpart, op, x, y, part + (int64_t)nb * Op::kSlots);
  return 3;
}

}  // namespace

Status katz_run(Ctx *ctx, const Graph *g, const gops_katz_config *cfg, double *scores, gops_run *run) {
  ctx->stats = gops_stats{};
  const int64_t n = g->n;
  *run = gops_run{0, 0.0, 1, 0};
  if (n == 0) return Status::ok();  // src/katz.rs:138-145
  cudaStream_t s = ctx->stream;
  Bufs b;
  LongPlan lp;
  GOPS_TRY(build_long_plan(s, g->in_rp, n, lp, false));
  const int nb = pull_blocks(n, lp);
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
    launches += pull(s, g->in_rp, g->in_col, n, lp, KatzOp{cfg->alpha, cfg->beta}, b.x, b.y, b.part);
    sum_blocks<<<1, kCThreads, 0, s>>>(b.part, nb, 1, b.sums);
    launches += 1;
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
  LongPlan lp;
  GOPS_TRY(build_long_plan(s, g->out_rp, n, lp, true));
  const int nb = pull_blocks(n, lp);
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
    launches += pull(s, g->out_rp, g->out_col, n, lp, EigOp{}, b.x, b.y, b.part);
    sum_blocks<<<1, kCThreads, 0, s>>>(b.part, nb, 2, b.sums);
    eig_scale<<<nbs, kCThreads, 0, s>>>(n, b.sums, b.x, b.y, b.part);
    sum_blocks<<<1, kCThreads, 0, s>>>(b.part, nbs, 1, b.sums);
    launches += 3;
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
  LongPlan lpi, lpo;
  GOPS_TRY(build_long_plan(s, g->in_rp, n, lpi, false));
  GOPS_TRY(build_long_plan(s, g->out_rp, n, lpo, true));
  const int nbi = pull_blocks(n, lpi), nbo = pull_blocks(n, lpo), nbs = blocks_for(n, 256, kCBlocks);
  const int nb = std::max(nbi, nbo);
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
    launches += pull(s, g->in_rp, g->in_col, n, lpi, SumOp{}, h.hub_r, h.nauth_r, h.part);
    sum_blocks<<<1, kCThreads, 0, s>>>(h.part, nbi, 1, h.sums);
    l2_scale<<<nbs, kCThreads, 0, s>>>(n, h.sums, h.auth, g->perm, h.nauth_r, h.part);
    sum_blocks<<<1, kCThreads, 0, s>>>(h.part, nbs, 1, h.sums + 2);
    unpermute_f64<<<blocks_for(n, 256, 4096), 256, 0, s>>>(h.nauth_r, g->perm, n, h.nauth);
    // hub: pull over the out-adjacency (original order)
    launches += pull(s, g->out_rp, g->out_col, n, lpo, SumOp{}, h.nauth, h.nhub, h.part);
    sum_blocks<<<1, kCThreads, 0, s>>>(h.part, nbo, 1, h.sums);
    l2_scale<<<nbs, kCThreads, 0, s>>>(n, h.sums, h.hub, nullptr, h.nhub, h.part);
    sum_blocks<<<1, kCThreads, 0, s>>>(h.part, nbs, 1, h.sums + 3);
    launches += 8;
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
