// The extern "C" entry points declared in include/gops.h.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <mutex>
#include <new>

#include "objects.cuh"

namespace gops {
Status solve(Ctx *ctx, Graph *g, const gops_config *cfg, int mode, const double *p_host,
             double *scores_host, gops_run *run);
Status dense_to_out_csr_device(Ctx *ctx, int64_t n, const double *d_M, int64_t **d_rp,
                               int32_t **d_col, double **d_w, int64_t *m_out);
Status edges_to_out_csr_device(Ctx *ctx, int64_t n, int64_t m, const int32_t *d_src, const int32_t *d_dst,
                               const double *d_w, int64_t **d_rp, int32_t **d_col, double **d_wout);
Status ppr_batch(Ctx *ctx, Graph *g, const gops_config *cfg, int64_t nsets, const int64_t *seed_ptr,
                 const int32_t *seed_idx, const float *x0, bool x0_on_device, float *scores,
                 bool scores_on_device, gops_run *runs, const double *r1_max, int32_t *rejected);
Status batch_set_tile(Ctx *ctx, Graph *g, int cols, int chunk, int l2_hints);
Status batch_get_tile(Graph *g, int *cols, int *chunk, int *l2_hints, float *cost);

constexpr int kMaxDevices = 64;
static std::mutex g_pool_mu;
static cudaMemPool_t g_pool[kMaxDevices] = {};
static bool g_pool_tried[kMaxDevices] = {};

cudaMemPool_t library_pool(int device) {
  if (device < 0 || device >= kMaxDevices) return nullptr;
  std::lock_guard<std::mutex> lock(g_pool_mu);
  if (!g_pool_tried[device]) {
    g_pool_tried[device] = true;
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    cudaMemPool_t pool = nullptr;
    if (cudaMemPoolCreate(&pool, &props) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) == cudaSuccess)
        g_pool[device] = pool;
      else
        cudaMemPoolDestroy(pool);
    }
    cudaGetLastError();  // a failed creation leaves the default pool in use
  }
  return g_pool[device];
}

static std::atomic<int64_t> g_alloc_fail_after{-1};  // < 0: no injection

bool alloc_fault_injected() {
  int64_t k = g_alloc_fail_after.load(std::memory_order_relaxed);
  while (k > 0) {  // this allocation still succeeds
    if (g_alloc_fail_after.compare_exchange_weak(k, k - 1, std::memory_order_relaxed)) return false;
  }
  return k == 0;
}

void library_pool_trim(int device) {
  if (device < 0 || device >= kMaxDevices) return;
  std::lock_guard<std::mutex> lock(g_pool_mu);
  if (g_pool[device]) cudaMemPoolTrimTo(g_pool[device], 0);
}
}  // namespace gops

using namespace gops;


namespace {

int write_msg(char *msg, size_t cap, const char *text) {
  if (msg && cap) std::snprintf(msg, cap, "%s", text);
  return GOPS_ERR_INVALID;
}

// Scalar checks on the host; the per-row and per-edge checks run on the
// device after the upload (csr_checks), before anything reads the arrays.
Status check_csr_host(int64_t n, const int64_t *row_ptr, const int32_t *col) {
  if (n < 0 || n >= INT32_MAX) return Status{GOPS_ERR_INVALID, "node count out of range"};
  if (!row_ptr) return Status{GOPS_ERR_INVALID, "row_ptr is NULL"};
  if (row_ptr[0] != 0) return Status{GOPS_ERR_INVALID, "row_ptr[0] must be 0"};
  const int64_t m = row_ptr[n];
  if (m < 0) return Status{GOPS_ERR_INVALID, "row_ptr must be non-decreasing"};
  if (m >= INT32_MAX) return Status{GOPS_ERR_INVALID, "edge count out of range"};
  if (m > 0 && !col) return Status{GOPS_ERR_INVALID, "col is NULL"};
  return Status::ok();
}

// flags[0]: some row_ptr[u+1] < row_ptr[u]; flags[1]: some col outside [0, n)
__global__ void csr_checks(int64_t n, const int64_t *rp, int64_t m, const int32_t *col, int *flags) {
  int bad_rp = 0, bad_col = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += stride)
    bad_rp |= rp[u + 1] < rp[u];
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += stride)
    bad_col |= (col[e] < 0) | (col[e] >= n);
  if (__any_sync(0xffffffffu, bad_rp) && (threadIdx.x & 31) == 0) atomicOr(&flags[0], 1);
  if (__any_sync(0xffffffffu, bad_col) && (threadIdx.x & 31) == 0) atomicOr(&flags[1], 1);
}

Status upload_impl(Ctx *ctx, int64_t n, const int64_t *row_ptr, const int32_t *col,
                   const double *w, Graph *g) {
  GOPS_TRY(check_csr_host(n, row_ptr, col));
  const int64_t m = row_ptr[n];
  g->n = n;
  g->m = m;
  cudaStream_t s = ctx->stream;
  int64_t *d_rp = nullptr;
  int32_t *d_col = nullptr;
  double *d_w = nullptr;
  Status st;
  auto fail = [&](cudaError_t e, const char *what) {
    return Status{e == cudaErrorMemoryAllocation ? GOPS_ERR_OOM : GOPS_ERR_CUDA,
                  std::string(what) + ": " + cudaGetErrorString(e)};
  };
  cudaError_t e = dev_malloc_async((void **)&d_rp, sizeof(int64_t) * (n + 1), s);
  if (e == cudaSuccess) e = dev_malloc_async((void **)&d_col, sizeof(int32_t) * (m > 0 ? m : 1), s);
  if (e == cudaSuccess && w) e = dev_malloc_async((void **)&d_w, sizeof(double) * (m > 0 ? m : 1), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_rp, row_ptr, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && m > 0) e = cudaMemcpyAsync(d_col, col, sizeof(int32_t) * m, cudaMemcpyHostToDevice, s);
  // the weights (the largest array) follow on the copy stream while the
  // checks and the edge sort, which do not read them, run on the main stream
  bool w_async = false;
  if (e == cudaSuccess && w && m > 0) {
    e = cudaEventRecord(ctx->copy_ev[0], s);  // after d_w's allocation and the column copy
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->copy_stream, ctx->copy_ev[0], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_w, w, sizeof(double) * m, cudaMemcpyHostToDevice, ctx->copy_stream);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->copy_ev[1], ctx->copy_stream);
    w_async = e == cudaSuccess;
  }
  if (e != cudaSuccess) st = fail(e, "graph upload");
  else {
    ctx->stats.h2d_bytes += sizeof(int64_t) * (n + 1) + sizeof(int32_t) * m + (w ? sizeof(double) * m : 0);
    // the same checks (and messages, in the same order) the host would make
    int *d_flags = nullptr;
    int flags[2] = {0, 0};
    e = dev_malloc_async((void **)&d_flags, sizeof(int) * 2, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_flags, 0, sizeof(int) * 2, s);
    if (e == cudaSuccess) {
      csr_checks<<<blocks_for(std::max(n, m), 256, ctx->num_sms * 8), 256, 0, s>>>(n, d_rp, m, d_col, d_flags);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(flags, d_flags, sizeof(int) * 2, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    free_async(d_flags, s);
    if (e != cudaSuccess) st = fail(e, "graph upload");
    else if (flags[0]) st = Status{GOPS_ERR_INVALID, "row_ptr must be non-decreasing"};
    else if (flags[1]) st = Status{GOPS_ERR_INVALID, "neighbor index out of range"};
    else st = graph_build_from_out_csr_device(ctx, g, d_rp, d_col, d_w, w_async ? ctx->copy_ev[1] : nullptr);
  }
  // every path: the main stream passes the weight copy before d_w is freed
  if (w_async) cudaStreamWaitEvent(s, ctx->copy_ev[1], 0);
  if (st.code == GOPS_OK) {  // kept: the out-adjacency drives eigenvector centrality
    g->out_rp = d_rp;
    g->out_col = d_col;
  } else {
    free_async(d_rp, s);
    free_async(d_col, s);
  }
  free_async(d_w, s);
  cudaError_t e2 = cudaStreamSynchronize(s);
  if (st.code == GOPS_OK && e2 != cudaSuccess) st = fail(e2, "graph upload");
  return st;
}

}  // namespace

extern "C" {

int gops_abi_version(void) { return GOPS_ABI_VERSION; }

int gops_debug_fail_allocations_after(int64_t count) {
  g_alloc_fail_after.store(count < 0 ? -1 : count, std::memory_order_relaxed);
  return GOPS_OK;
}

int gops_ctx_create(int device, gops_ctx **out) {
  if (!out) return GOPS_ERR_INVALID;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return GOPS_ERR_NO_DEVICE;
  if (device < 0 || device >= count) return GOPS_ERR_INVALID;
  gops_ctx *c = new (std::nothrow) gops_ctx();
  if (!c) return GOPS_ERR_OOM;
  Ctx &x = c->impl;
  x.device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&x.num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&x.stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMallocHost((void **)&x.host_state, sizeof(SolveState));
  for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaEventCreate(&x.ev[i]);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&x.copy_stream, cudaStreamNonBlocking);
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&x.copy_ev[i], cudaEventDisableTiming);
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&x.build_ev[i], cudaEventDisableTiming);
  if (e != cudaSuccess) {
    gops_ctx_destroy(c);
    return e == cudaErrorMemoryAllocation ? GOPS_ERR_OOM : GOPS_ERR_CUDA;
  }
  // the no-allocation entry point's scratch array: mapped on this device now
  const Status na = noalloc_attach(device);
  if (na.code != GOPS_OK) {
    gops_ctx_destroy(c);
    return na.code;
  }
  x.noalloc_attached = true;
  *out = c;
  return GOPS_OK;
}

void gops_ctx_destroy(gops_ctx *ctx) {
  if (!ctx) return;
  Ctx &x = ctx->impl;
  cudaSetDevice(x.device);
  if (x.stream) cudaStreamSynchronize(x.stream);
  for (int i = 0; i < 4; ++i)
    if (x.ev[i]) cudaEventDestroy(x.ev[i]);
  if (x.copy_stream) cudaStreamSynchronize(x.copy_stream);
  for (int i = 0; i < 2; ++i)
    if (x.copy_ev[i]) cudaEventDestroy(x.copy_ev[i]);
  for (int i = 0; i < 2; ++i)
    if (x.build_ev[i]) cudaEventDestroy(x.build_ev[i]);
  for (int i = 0; i < 2; ++i) {
    if (x.hstage[i]) cudaFreeHost(x.hstage[i]);
    if (x.sev[i]) cudaEventDestroy(x.sev[i]);
  }
  if (x.copy_stream) cudaStreamDestroy(x.copy_stream);
  if (x.host_state) cudaFreeHost(x.host_state);
  for (cudaEvent_t e : x.tev) cudaEventDestroy(e);
  if (x.stream) cudaStreamDestroy(x.stream);
  library_pool_trim(x.device);  // memory that no live graph or model holds
  if (x.noalloc_attached) noalloc_detach(x.device);
  delete ctx;
}

const char *gops_last_error(const gops_ctx *ctx) {
  return ctx ? ctx->impl.last_error.c_str() : "null context";
}

int gops_ctx_stats(const gops_ctx *ctx, gops_stats *out) {
  if (!ctx || !out) return GOPS_ERR_INVALID;
  *out = ctx->impl.stats;
  return GOPS_OK;
}

void *gops_ctx_stream(gops_ctx *ctx) { return ctx ? (void *)ctx->impl.stream : nullptr; }

int gops_ctx_set_timing(gops_ctx *ctx, int enable) {
  if (!ctx) return GOPS_ERR_INVALID;
  ctx->impl.timing = enable != 0;
  return GOPS_OK;
}

int gops_config_validate(const gops_config *cfg, char *msg, size_t cap) {
  if (!cfg) return write_msg(msg, cap, "config is NULL");
  if (!std::isfinite(cfg->damping)) return write_msg(msg, cap, "damping must be finite");
  if (!(cfg->damping >= 0.0 && cfg->damping <= 1.0)) return write_msg(msg, cap, "damping must be in [0,1]");
  if (cfg->max_iterations == 0) return write_msg(msg, cap, "max_iterations must be > 0");
  if (!std::isfinite(cfg->tolerance) || cfg->tolerance <= 0.0)
    return write_msg(msg, cap, "tolerance must be finite and > 0");
  return GOPS_OK;
}

int gops_weights_validate(int64_t m, const double *w, char *msg, size_t cap) {
  for (int64_t e = 0; e < m; ++e) {
    if (!std::isfinite(w[e])) return write_msg(msg, cap, "edge weights must be finite");
    if (w[e] < 0.0) return write_msg(msg, cap, "edge weights must be non-negative");
  }
  return GOPS_OK;
}

int gops_personalization_validate(int64_t node_count, int64_t len, const double *p, char *msg,
                                  size_t cap) {
  if (len != node_count) {
    char buf[160];
    std::snprintf(buf, sizeof buf,
                  "personalization length must equal node_count (len=%lld node_count=%lld)",
                  (long long)len, (long long)node_count);
    return write_msg(msg, cap, buf);
  }
  for (int64_t i = 0; i < len; ++i) {
    if (!std::isfinite(p[i])) return write_msg(msg, cap, "personalization entries must be finite");
    if (p[i] < 0.0) return write_msg(msg, cap, "personalization entries must be non-negative");
  }
  double s = 0.0;
  for (int64_t i = 0; i < len; ++i) s += p[i];
  if (s <= 0.0) return write_msg(msg, cap, "personalization sum must be > 0");
  return GOPS_OK;
}

int gops_graph_upload(gops_ctx *ctx, int64_t n, const int64_t *row_ptr, const int32_t *col,
                      const double *weights, gops_graph **out) {
  if (!ctx || !out) return GOPS_ERR_INVALID;
  *out = nullptr;
  Ctx &c = ctx->impl;
  cudaSetDevice(c.device);
  c.stats = gops_stats{};
  gops_graph *g = new (std::nothrow) gops_graph();
  if (!g) return c.set(Status{GOPS_ERR_OOM, "host allocation failed"});
  g->impl.ctx = &c;
  g->impl.device = c.device;
  Status st = upload_impl(&c, n, row_ptr, col, weights, &g->impl);
  if (st.code != GOPS_OK) {
    graph_free_device(g->impl);
    delete g;
    return c.set(st);
  }
  *out = g;
  return GOPS_OK;
}

int gops_graph_from_dense(gops_ctx *ctx, int64_t n, const double *matrix, gops_graph **out) {
  if (!ctx || !out) return GOPS_ERR_INVALID;
  *out = nullptr;
  Ctx &c = ctx->impl;
  cudaSetDevice(c.device);
  c.stats = gops_stats{};
  if (n < 0 || n >= 46341) return c.set(Status{GOPS_ERR_INVALID, "dense matrix too large"});
  if (n > 0 && !matrix) return c.set(Status{GOPS_ERR_INVALID, "matrix is NULL"});
  gops_graph *g = new (std::nothrow) gops_graph();
  if (!g) return c.set(Status{GOPS_ERR_OOM, "host allocation failed"});
  g->impl.ctx = &c;
  g->impl.device = c.device;
  cudaStream_t s = c.stream;
  double *d_M = nullptr, *d_w = nullptr;
  int64_t *d_rp = nullptr;
  int32_t *d_col = nullptr;
  int64_t m = 0;
  Status st;
  const size_t bytes = sizeof(double) * (size_t)std::max<int64_t>(n * n, 1);
  cudaError_t e = dev_malloc_async((void **)&d_M, bytes, s);
  if (e == cudaSuccess && n > 0) e = cudaMemcpyAsync(d_M, matrix, sizeof(double) * (size_t)(n * n), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) st = Status{e == cudaErrorMemoryAllocation ? GOPS_ERR_OOM : GOPS_ERR_CUDA,
                                    std::string("dense upload: ") + cudaGetErrorString(e)};
  if (st.code == GOPS_OK) {
    c.stats.h2d_bytes += sizeof(double) * (size_t)(n * n);
    st = dense_to_out_csr_device(&c, n, d_M, &d_rp, &d_col, &d_w, &m);
  }
  if (st.code == GOPS_OK && m >= INT32_MAX) st = Status{GOPS_ERR_INVALID, "edge count out of range"};
  if (st.code == GOPS_OK) {
    g->impl.n = n;
    g->impl.m = m;
    st = graph_build_from_out_csr_device(&c, &g->impl, d_rp, d_col, d_w);
  }
  free_async(d_M, s);
  if (st.code == GOPS_OK) {
    g->impl.out_rp = d_rp;
    g->impl.out_col = d_col;
  } else {
    free_async(d_rp, s);
    free_async(d_col, s);
  }
  free_async(d_w, s);
  cudaStreamSynchronize(s);
  if (st.code != GOPS_OK) {
    graph_free_device(g->impl);
    delete g;
    return c.set(st);
  }
  *out = g;
  return GOPS_OK;
}

int gops_graph_from_edges(gops_ctx *ctx, int64_t n, int64_t m, const int32_t *src, const int32_t *dst,
                          const double *weights, gops_graph **out) {
  if (!ctx || !out) return GOPS_ERR_INVALID;
  *out = nullptr;
  Ctx &c = ctx->impl;
  cudaSetDevice(c.device);
  c.stats = gops_stats{};
  if (n < 0 || n >= INT32_MAX) return c.set(Status{GOPS_ERR_INVALID, "node count out of range"});
  if (m < 0 || m >= INT32_MAX) return c.set(Status{GOPS_ERR_INVALID, "edge count out of range"});
  if (m > 0 && (!src || !dst)) return c.set(Status{GOPS_ERR_INVALID, "edge list is NULL"});
  if (m > 0 && n == 0) return c.set(Status{GOPS_ERR_INVALID, "edge endpoint out of range"});
  gops_graph *g = new (std::nothrow) gops_graph();
  if (!g) return c.set(Status{GOPS_ERR_OOM, "host allocation failed"});
  g->impl.ctx = &c;
  g->impl.device = c.device;
  cudaStream_t s = c.stream;
  int32_t *d_src = nullptr, *d_dst = nullptr;
  double *d_w = nullptr, *d_wout = nullptr;
  int64_t *d_rp = nullptr;
  int32_t *d_col = nullptr;
  const size_t mm = (size_t)std::max<int64_t>(m, 1);
  cudaError_t e = dev_malloc_async((void **)&d_src, sizeof(int32_t) * mm, s);
  if (e == cudaSuccess) e = dev_malloc_async((void **)&d_dst, sizeof(int32_t) * mm, s);
  if (e == cudaSuccess && weights) e = dev_malloc_async((void **)&d_w, sizeof(double) * mm, s);
  if (e == cudaSuccess && m > 0) e = cudaMemcpyAsync(d_src, src, sizeof(int32_t) * m, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && m > 0) e = cudaMemcpyAsync(d_dst, dst, sizeof(int32_t) * m, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && weights && m > 0)
    e = cudaMemcpyAsync(d_w, weights, sizeof(double) * m, cudaMemcpyHostToDevice, s);
  Status st;
  if (e != cudaSuccess)
    st = Status{e == cudaErrorMemoryAllocation ? GOPS_ERR_OOM : GOPS_ERR_CUDA,
                std::string("edge list upload: ") + cudaGetErrorString(e)};
  if (st.code == GOPS_OK) {
    c.stats.h2d_bytes += (2 * sizeof(int32_t) + (weights ? sizeof(double) : 0)) * (size_t)m;
    st = edges_to_out_csr_device(&c, n, m, d_src, d_dst, d_w, &d_rp, &d_col, &d_wout);
  }
  if (st.code == GOPS_OK) {
    g->impl.n = n;
    g->impl.m = m;
    st = graph_build_from_out_csr_device(&c, &g->impl, d_rp, d_col, d_wout);
  }
  free_async(d_src, s);
  free_async(d_dst, s);
  free_async(d_w, s);
  if (st.code == GOPS_OK) {
    g->impl.out_rp = d_rp;
    g->impl.out_col = d_col;
  } else {
    free_async(d_rp, s);
    free_async(d_col, s);
  }
  free_async(d_wout, s);
  cudaStreamSynchronize(s);
  if (st.code != GOPS_OK) {
    graph_free_device(g->impl);
    delete g;
    return c.set(st);
  }
  *out = g;
  return GOPS_OK;
}

void gops_graph_destroy(gops_graph *g) {
  if (!g) return;
  // the context may already be gone: use the device recorded at upload
  // (cudaFree waits for the device's pending work before it frees)
  cudaSetDevice(g->impl.device);
  graph_free_device(g->impl);
  delete g;
}

int gops_graph_info(const gops_graph *g, int64_t *n, int64_t *m, int32_t *weighted) {
  if (!g) return GOPS_ERR_INVALID;
  if (n) *n = g->impl.n;
  if (m) *m = g->impl.m;
  if (weighted) *weighted = g->impl.weighted ? 1 : 0;
  return GOPS_OK;
}

static int run_common(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg, int mode,
                      const double *p, double *scores, gops_run *run) {
  if (!ctx) return GOPS_ERR_INVALID;
  Ctx &c = ctx->impl;
  if (!g || !cfg || !run) return c.set(Status{GOPS_ERR_INVALID, "null argument"});
  if (g->impl.ctx != &c) return c.set(Status{GOPS_ERR_INVALID, "graph belongs to another context"});
  if (mode == 2 && g->impl.n > 0 && !p) return c.set(Status{GOPS_ERR_INVALID, "personalization is NULL"});
  cudaSetDevice(c.device);
  return c.set(solve(&c, const_cast<Graph *>(&g->impl), cfg, mode, p, scores, run));
}

int gops_pagerank_run(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg, double *scores,
                      gops_run *run) {
  return run_common(ctx, g, cfg, 0, nullptr, scores, run);
}

int gops_pagerank_weighted_run(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg,
                               double *scores, gops_run *run) {
  return run_common(ctx, g, cfg, 1, nullptr, scores, run);
}

int gops_personalized_pagerank_run(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg,
                                   const double *personalization, double *scores, gops_run *run) {
  return run_common(ctx, g, cfg, 2, personalization, scores, run);
}

static int batch_common(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg, int64_t nsets,
                        const int64_t *seed_ptr, const int32_t *seed_idx, const float *x0,
                        float *scores, gops_run *runs, bool on_device) {
  if (!ctx) return GOPS_ERR_INVALID;
  Ctx &c = ctx->impl;
  if (!g || !cfg || nsets < 0 || (nsets > 0 && (!seed_ptr || (!seed_idx && seed_ptr[nsets] > seed_ptr[0]))))
    return c.set(Status{GOPS_ERR_INVALID, "null argument"});
  if (g->impl.ctx != &c) return c.set(Status{GOPS_ERR_INVALID, "graph belongs to another context"});
  cudaSetDevice(c.device);
  return c.set(ppr_batch(&c, const_cast<Graph *>(&g->impl), cfg, nsets, seed_ptr, seed_idx, x0, on_device,
                         scores, on_device, runs, nullptr, nullptr));
}

int gops_ppr_batch(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg, int64_t nsets,
                   const int64_t *seed_ptr, const int32_t *seed_idx, const float *x0, float *scores,
                   gops_run *runs) {
  return batch_common(ctx, g, cfg, nsets, seed_ptr, seed_idx, x0, scores, runs, false);
}

int gops_ppr_batch_device(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg, int64_t nsets,
                          const int64_t *seed_ptr, const int32_t *seed_idx, const float *x0_device,
                          float *scores_device, gops_run *runs) {
  return batch_common(ctx, g, cfg, nsets, seed_ptr, seed_idx, x0_device, scores_device, runs, true);
}

int gops_ppr_batch_set_tile(gops_ctx *ctx, const gops_graph *g, int32_t cols, int32_t chunk, int32_t l2_hints) {
  if (!ctx) return GOPS_ERR_INVALID;
  Ctx &c = ctx->impl;
  if (!g) return c.set(Status{GOPS_ERR_INVALID, "null argument"});
  if (g->impl.ctx != &c) return c.set(Status{GOPS_ERR_INVALID, "graph belongs to another context"});
  if (g->impl.n == 0) return GOPS_OK;
  cudaSetDevice(c.device);
  return c.set(batch_set_tile(&c, const_cast<Graph *>(&g->impl), cols, chunk, l2_hints));
}

int gops_ppr_batch_tile(const gops_graph *g, int32_t *cols, int32_t *chunk, int32_t *l2_hints, float *cost) {
  if (!g || !cols || !chunk || !l2_hints) return GOPS_ERR_INVALID;
  int c = 0, ch = 0, l2 = 0;
  batch_get_tile(const_cast<Graph *>(&g->impl), &c, &ch, &l2, cost);
  *cols = c;
  *chunk = ch;
  *l2_hints = l2;
  return GOPS_OK;
}

const double *gops_ctx_scores_device(const gops_ctx *ctx) {
  return ctx ? ctx->impl.last_scores : nullptr;
}

}  // extern "C"
