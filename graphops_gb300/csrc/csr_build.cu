// Graph ingestion on the device.
//
//  K1  out-adjacency (adapter order) -> in-edge CSR.  Per out-row: source ids,
//      out-degree, weight sum sum max(w,0) and transition weights
//      max(w,0)/sum (replacing the neighbor / out_wsum precompute of
//      src/pagerank.rs:136-137,226-234 and src/ppr.rs:112); then a stable radix
//      sort of edge ids by destination, so every in-row lists its sources in
//      ascending source order, the order the reference scatters in
//      (src/pagerank.rs:154-162).
//  K2  the pull kernels' work partition: runs of rows whose in-edges start in
//      the same W-edge window (so fewer than 2W in-edges, staged in shared
//      memory), at most kRowCap rows each; rows with more than W in-edges
//      ("hubs") are split into 2W-edge chunks.
//  Dense  AdjacencyMatrix (src/graph.rs:128-141) -> out-CSR by a warp-ballot
//      compaction of each matrix row (entries > 0.0, ascending column).
#include <algorithm>

#include "objects.cuh"
#include "primitives.cuh"

namespace gops {

constexpr int kRowCap = 256;  // rows per normal item (one epilogue thread each)

namespace {

__global__ void out_row_pass(int64_t n, const int64_t *__restrict__ rp, const int32_t *__restrict__ col,
                             const double *__restrict__ w, uint32_t *__restrict__ src,
                             float *__restrict__ val_out, float *__restrict__ deg_f,
                             uint32_t *__restrict__ dmask, unsigned long long *__restrict__ indeg) {
  const int lane = threadIdx.x & 31;
  const int64_t u = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (u >= n) return;
  const int64_t b = rp[u], e = rp[u + 1];
  if (lane == 0) deg_f[u] = (float)(e - b);
  for (int64_t i = b + lane; i < e; i += 32) {
    src[i] = (uint32_t)u;
    atomicAdd(&indeg[col[i]], 1ull);
  }
  if (w) {
    double s = 0.0;
    for (int64_t i = b + lane; i < e; i += 32) s += fmax(w[i], 0.0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const double inv = s > 0.0 ? 1.0 / s : 0.0;
    for (int64_t i = b + lane; i < e; i += 32) {
      const double wc = fmax(w[i], 0.0);
      val_out[i] = wc > 0.0 ? (float)(wc * inv) : 0.0f;
    }
    if (lane == 0 && s == 0.0) atomicOr(&dmask[u >> 5], 1u << (u & 31));
  }
}

__global__ void iota_u32(uint32_t *v, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    v[i] = (uint32_t)i;
}

__global__ void copy_keys(const int32_t *col, uint32_t *keys, int64_t m) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x)
    keys[i] = (uint32_t)col[i];
}

__global__ void gather_in_edges(const uint32_t *order, const uint32_t *src, const float *val_out,
                                int32_t *in_col, float *in_val, int64_t m) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t e = order[i];
    in_col[i] = (int32_t)src[e];
    if (in_val) in_val[i] = val_out[e];
  }
}

__device__ __forceinline__ bool is_long_row(const int64_t *rp, int64_t v, int W) {
  return rp[v + 1] - rp[v] > W;
}

__device__ __forceinline__ bool is_start(const int64_t *rp, int64_t v, int64_t n, int W) {
  if (v >= n) return true;
  if (v == 0 || (v % kRowCap) == 0) return true;
  if (is_long_row(rp, v, W) || is_long_row(rp, v - 1, W)) return true;
  return (rp[v] / W) != (rp[v - 1] / W);
}

__global__ void item_units(const int64_t *rp, int64_t n, int W, int64_t *units) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v <= n;
       v += (int64_t)gridDim.x * blockDim.x) {
    int64_t u = 0;
    if (v < n && is_start(rp, v, n, W)) {
      const int64_t d = rp[v + 1] - rp[v];
      u = d > W ? ceil_div<int64_t>(d, 2 * (int64_t)W) : 1;
    }
    units[v] = u;
  }
}

__global__ void item_fill(const int64_t *rp, int64_t n, int W, const int64_t *ibase, Item *items) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const bool lng = is_long_row(rp, v, W);
    if (is_start(rp, v, n, W)) {
      const int64_t b = ibase[v];
      if (lng) {
        const int64_t nch = ibase[v + 1] - b;
        for (int64_t c = 0; c < nch; ++c)
          items[b + c] = Item{(int32_t)v, (int32_t)(v + 1), (int32_t)b, (int32_t)nch};
      } else {
        items[b].r0 = (int32_t)v;
        items[b].first = -1;
        items[b].nchunks = 0;
      }
    }
    // the last row of a normal run closes it: its item is the one just
    // before the next start's items
    if (!lng && is_start(rp, v + 1, n, W)) items[ibase[v + 1] - 1].r1 = (int32_t)(v + 1);
  }
}

__global__ void max_chunks_kernel(const Item *items, int64_t n_items, int *out) {
  int best = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_items;
       i += (int64_t)gridDim.x * blockDim.x)
    best = max(best, items[i].nchunks);
  best = __reduce_max_sync(0xffffffffu, best);
  if ((threadIdx.x & 31) == 0) atomicMax(out, best);
}

// Dense matrix rows: count entries > 0 (pass 0) or write them in ascending
// column order (pass 1), one warp per row.
__global__ void dense_rows(int64_t n, const double *__restrict__ M, int64_t *counts,
                           const int64_t *rp, int32_t *col, double *w) {
  const int lane = threadIdx.x & 31;
  const int64_t u = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (u >= n) return;
  const double *row = M + u * n;
  int64_t pos = rp ? rp[u] : 0;
  int64_t cnt = 0;
  for (int64_t j0 = 0; j0 < n; j0 += 32) {
    const int64_t j = j0 + lane;
    const double x = j < n ? row[j] : 0.0;
    const bool edge = x > 0.0;
    const unsigned mask = __ballot_sync(0xffffffffu, edge);
    if (rp && edge) {
      const int64_t at = pos + cnt + __popc(mask & ((1u << lane) - 1u));
      col[at] = (int32_t)j;
      w[at] = x;
    }
    cnt += __popc(mask);
  }
  if (!rp && lane == 0) counts[u] = cnt;
}

int grid_for(int64_t work, int threads) {
  int64_t b = ceil_div<int64_t>(work, threads);
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, 1 << 20));
}

int bits_for(int64_t n) {
  int b = 0;
  while (b < 63 && ((int64_t)1 << b) < n) ++b;
  return b;
}

}  // namespace

Status graph_build_from_out_csr_device(Ctx *ctx, Graph *g, const int64_t *d_out_rp,
                                       const int32_t *d_out_col, const double *d_w) {
  cudaStream_t s = ctx->stream;
  const int64_t n = g->n, m = g->m;
  const int W = g->window > 0 ? g->window : 1024;
  g->window = W;
  g->weighted = d_w != nullptr;
  Status st;
  uint32_t *src = nullptr, *keys = nullptr, *vals = nullptr, *keys2 = nullptr, *vals2 = nullptr;
  float *val_out = nullptr;
  unsigned long long *indeg = nullptr;
  int64_t *units = nullptr;
  int *maxc = nullptr;
  auto cleanup = [&]() {
    free_async(src, s); free_async(keys, s); free_async(vals, s);
    free_async(keys2, s); free_async(vals2, s); free_async(val_out, s);
    free_async(indeg, s); free_async(units, s); free_async(maxc, s);
  };
#define BUILD_TRY(expr)                                                                     \
  do {                                                                                      \
    cudaError_t _e = (expr);                                                                \
    if (_e != cudaSuccess) {                                                                \
      cleanup();                                                                            \
      return Status{_e == cudaErrorMemoryAllocation ? GOPS_ERR_OOM : GOPS_ERR_CUDA,         \
                    std::string("graph build: ") + #expr + ": " + cudaGetErrorString(_e)}; \
    }                                                                                       \
  } while (0)
  const size_t mm = (size_t)std::max<int64_t>(m, 1);
  BUILD_TRY(cudaMalloc(&g->in_rp, sizeof(int64_t) * (n + 1)));
  BUILD_TRY(cudaMalloc(&g->in_col, sizeof(int32_t) * mm));
  BUILD_TRY(cudaMalloc(&g->deg, sizeof(float) * std::max<int64_t>(n, 1)));
  if (g->weighted) {
    BUILD_TRY(cudaMalloc(&g->in_val, sizeof(float) * mm));
    BUILD_TRY(cudaMalloc(&g->dmask_w, sizeof(uint32_t) * (size_t)(n / 32 + 1)));
    BUILD_TRY(cudaMemsetAsync(g->dmask_w, 0, sizeof(uint32_t) * (size_t)(n / 32 + 1), s));
    BUILD_TRY(cudaMallocAsync((void **)&val_out, sizeof(float) * mm, s));
  }
  BUILD_TRY(cudaMallocAsync((void **)&src, sizeof(uint32_t) * mm, s));
  BUILD_TRY(cudaMallocAsync((void **)&indeg, sizeof(unsigned long long) * (n + 1), s));
  BUILD_TRY(cudaMemsetAsync(indeg, 0, sizeof(unsigned long long) * (n + 1), s));
  if (n > 0) {
    out_row_pass<<<(unsigned)ceil_div<int64_t>(n, 8), 256, 0, s>>>(
        n, d_out_rp, d_out_col, d_w, src, val_out, g->deg, g->dmask_w, indeg);
    BUILD_TRY(cudaGetLastError());
  }
  // in_rp = exclusive scan of in-degrees (entry n is 0, so in_rp[n] == m)
  st = exclusive_scan_i64((const int64_t *)indeg, g->in_rp, n + 1, s);
  if (st.code != GOPS_OK) { cleanup(); return st; }
  if (m > 0) {
    BUILD_TRY(cudaMallocAsync((void **)&keys, sizeof(uint32_t) * mm, s));
    BUILD_TRY(cudaMallocAsync((void **)&vals, sizeof(uint32_t) * mm, s));
    BUILD_TRY(cudaMallocAsync((void **)&keys2, sizeof(uint32_t) * mm, s));
    BUILD_TRY(cudaMallocAsync((void **)&vals2, sizeof(uint32_t) * mm, s));
    copy_keys<<<grid_for(m, 256), 256, 0, s>>>(d_out_col, keys, m);
    iota_u32<<<grid_for(m, 256), 256, 0, s>>>(vals, m);
    BUILD_TRY(cudaGetLastError());
    bool alt = false;
    st = radix_sort_pairs_u32(keys, vals, keys2, vals2, m, bits_for(n), &alt, s);
    if (st.code != GOPS_OK) { cleanup(); return st; }
    gather_in_edges<<<grid_for(m, 256), 256, 0, s>>>(alt ? vals2 : vals, src, val_out, g->in_col,
                                                     g->in_val, m);
    BUILD_TRY(cudaGetLastError());
  }
  // K2: work items
  BUILD_TRY(cudaMallocAsync((void **)&units, sizeof(int64_t) * (n + 1), s));
  item_units<<<grid_for(n + 1, 256), 256, 0, s>>>(g->in_rp, n, W, units);
  BUILD_TRY(cudaGetLastError());
  st = exclusive_scan_i64(units, units, n + 1, s);
  if (st.code != GOPS_OK) { cleanup(); return st; }
  int64_t n_items = 0;
  BUILD_TRY(cudaMemcpyAsync(&n_items, units + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  BUILD_TRY(cudaStreamSynchronize(s));
  if (n_items >= INT32_MAX) { cleanup(); return Status{GOPS_ERR_INVALID, "graph too large"}; }
  g->n_items = (int32_t)n_items;
  BUILD_TRY(cudaMalloc(&g->items, sizeof(Item) * std::max<int64_t>(n_items, 1)));
  if (n > 0) {
    item_fill<<<grid_for(n, 256), 256, 0, s>>>(g->in_rp, n, W, units, g->items);
    BUILD_TRY(cudaGetLastError());
  }
  BUILD_TRY(cudaMallocAsync((void **)&maxc, sizeof(int), s));
  BUILD_TRY(cudaMemsetAsync(maxc, 0, sizeof(int), s));
  if (n_items > 0) {
    max_chunks_kernel<<<grid_for(n_items, 256), 256, 0, s>>>(g->items, n_items, maxc);
    BUILD_TRY(cudaGetLastError());
  }
  int mc = 0;
  BUILD_TRY(cudaMemcpyAsync(&mc, maxc, sizeof(int), cudaMemcpyDeviceToHost, s));
  BUILD_TRY(cudaStreamSynchronize(s));
  g->max_chunks = mc;
  cleanup();
  return Status::ok();
#undef BUILD_TRY
}

// Dense AdjacencyMatrix -> device out-CSR -> the build above.
Status dense_to_out_csr_device(Ctx *ctx, int64_t n, const double *d_M, int64_t **d_rp,
                               int32_t **d_col, double **d_w, int64_t *m_out) {
  cudaStream_t s = ctx->stream;
  *d_rp = nullptr; *d_col = nullptr; *d_w = nullptr;
  GOPS_CUDA_TRY(cudaMallocAsync((void **)d_rp, sizeof(int64_t) * (n + 1), s));
  GOPS_CUDA_TRY(cudaMemsetAsync(*d_rp, 0, sizeof(int64_t) * (n + 1), s));
  if (n > 0) {
    dense_rows<<<(unsigned)ceil_div<int64_t>(n, 8), 256, 0, s>>>(n, d_M, *d_rp, nullptr, nullptr,
                                                                 nullptr);
    GOPS_CUDA_TRY(cudaGetLastError());
  }
  GOPS_TRY(exclusive_scan_i64(*d_rp, *d_rp, n + 1, s));
  int64_t m = 0;
  GOPS_CUDA_TRY(cudaMemcpyAsync(&m, *d_rp + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  *m_out = m;
  GOPS_CUDA_TRY(cudaMallocAsync((void **)d_col, sizeof(int32_t) * std::max<int64_t>(m, 1), s));
  GOPS_CUDA_TRY(cudaMallocAsync((void **)d_w, sizeof(double) * std::max<int64_t>(m, 1), s));
  if (n > 0 && m > 0) {
    dense_rows<<<(unsigned)ceil_div<int64_t>(n, 8), 256, 0, s>>>(n, d_M, nullptr, *d_rp, *d_col,
                                                                 *d_w);
    GOPS_CUDA_TRY(cudaGetLastError());
  }
  return Status::ok();
}

}  // namespace gops
