// gops_pagerank_run_noalloc: plain PageRank without any allocation.
//
// Some callers cannot allocate device memory at the moment they need a
// solve: a process whose device memory is owned by another allocator (a
// framework's caching pool holds the rest of the GPU, so a cudaMalloc here
// could fail or force that pool to release its cache), or a latency-critical
// path where cudaMalloc / cudaFree would synchronize the device.  For them
// this entry point runs the same kernels as gops_pagerank_run on a scratch
// area that is a file-scope __device__ array of fixed size, instead of the
// graph's lazily allocated workspace.  The graph itself must already be on
// the device (gops_graph_upload / gops_graph_from_dense, which do allocate,
// typically once at start-up).
//
// Limits: at most kNoAllocMaxNodes nodes and kNoAllocMaxHubTasks hub tasks;
// larger graphs are rejected with GOPS_ERR_INVALID.  The array (about 13 MB)
// is held by every GPU that uses this library until the process exits.
// With CUDA's lazy module loading the array's memory is committed only when
// this file's module is first loaded on a device, so gops_ctx_create loads
// it: it looks up the array's device address (cudaGetSymbolAddress, with the
// device current) for the context's device, and the no-alloc calls that
// follow need no device memory of their own.  The cached address is dropped
// when the last context on the device is destroyed and looked up again by
// the next gops_ctx_create; a device reset while a context lives
// invalidates it, like every other device object of the library.
// Every call shares the array and it keeps the last call's contents; the
// solve clears what must start at zero.  Calls that overlap on the GPU (from
// two contexts or streams at once) race on it and must be serialized by the
// caller.  After a no-alloc call, gops_ctx_scores_device points into the
// array: the next no-alloc call on that device, from any context,
// overwrites those scores.
#include <cstdio>
#include <mutex>

#include "objects.cuh"

namespace gops {
namespace {

constexpr int64_t kNoAllocMaxNodes = 1 << 18;     // 262,144
constexpr int64_t kNoAllocMaxHubTasks = 1 << 16;  // 65,536

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// byte offsets of the workspace arrays inside the scratch array
struct Layout {
  size_t gdf0, gdf1, gf0, gf1, acc, tail, scores, lpart, lcnt, state, sums, total;
};

constexpr Layout make_layout() {
  Layout l{};
  const size_t nv = (size_t)kNoAllocMaxNodes + 1;  // gathered vectors: entry n is padding
  const size_t nn = (size_t)kNoAllocMaxNodes;
  size_t o = 0;
  l.gdf0 = o; o = align256(o + sizeof(float2) * nv);
  l.gdf1 = o; o = align256(o + sizeof(float2) * nv);
  l.gf0 = o; o = align256(o + sizeof(float) * nv);
  l.gf1 = o; o = align256(o + sizeof(float) * nv);
  l.acc = o; o = align256(o + sizeof(float2) * nn);
  l.tail = o; o = align256(o + sizeof(float) * nn);
  l.scores = o; o = align256(o + sizeof(double) * nn);
  l.lpart = o; o = align256(o + sizeof(float2) * (size_t)kNoAllocMaxHubTasks);
  l.lcnt = o; o = align256(o + sizeof(unsigned) * nn);
  l.state = o; o = align256(o + sizeof(SolveState));
  l.sums = o; o = align256(o + sizeof(long long) * 12);
  l.total = o;
  return l;
}

constexpr Layout kLayout = make_layout();

__device__ __align__(256) unsigned char g_noalloc_scratch[kLayout.total];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char *g_scratch_addr[kMaxDevices] = {};
int g_live_contexts[kMaxDevices] = {};

// Device address of the scratch array on `device` (which must be current),
// looked up once per device and cached.  The caller holds g_mu.
Status scratch_address_locked(int device, unsigned char **out) {
  if (device < 0 || device >= kMaxDevices) return Status{GOPS_ERR_INVALID, "device index out of range"};
  if (!g_scratch_addr[device]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return Status{e == cudaErrorMemoryAllocation ? GOPS_ERR_OOM : GOPS_ERR_CUDA,
                    std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)};
    g_scratch_addr[device] = static_cast<unsigned char *>(p);
  }
  *out = g_scratch_addr[device];
  return Status::ok();
}

Workspace workspace_in(unsigned char *base) {
  Workspace ws;
  ws.n = kNoAllocMaxNodes;
  ws.gdf[0] = reinterpret_cast<float2 *>(base + kLayout.gdf0);
  ws.gdf[1] = reinterpret_cast<float2 *>(base + kLayout.gdf1);
  ws.gf[0] = reinterpret_cast<float *>(base + kLayout.gf0);
  ws.gf[1] = reinterpret_cast<float *>(base + kLayout.gf1);
  ws.acc = reinterpret_cast<float2 *>(base + kLayout.acc);
  ws.tail = reinterpret_cast<float *>(base + kLayout.tail);
  ws.pdf = nullptr;  // personalization is not used by plain PageRank
  ws.scores = reinterpret_cast<double *>(base + kLayout.scores);
  ws.lpart = reinterpret_cast<float2 *>(base + kLayout.lpart);
  ws.lcnt = reinterpret_cast<unsigned *>(base + kLayout.lcnt);
  ws.state = reinterpret_cast<SolveState *>(base + kLayout.state);
  ws.sums = reinterpret_cast<long long *>(base + kLayout.sums);
  return ws;
}

}  // namespace

// Called by gops_ctx_create with `device` current: loads this file's module
// on the device (committing the array's memory) and caches its address.
Status noalloc_attach(int device) {
  std::lock_guard<std::mutex> lock(g_mu);
  unsigned char *base = nullptr;
  GOPS_TRY(scratch_address_locked(device, &base));
  ++g_live_contexts[device];
  return Status::ok();
}

// Called by gops_ctx_destroy: the last context on a device drops the cached
// address, so a context created after a device reset looks it up again.
void noalloc_detach(int device) {
  if (device < 0 || device >= kMaxDevices) return;
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_live_contexts[device] > 0 && --g_live_contexts[device] == 0) g_scratch_addr[device] = nullptr;
}

}  // namespace gops

using namespace gops;

extern "C" int gops_pagerank_run_noalloc(gops_ctx *ctx, const gops_graph *g, const gops_config *cfg,
                                         double *scores, gops_run *run) {
  if (!ctx) return GOPS_ERR_INVALID;
  Ctx &c = ctx->impl;
  if (!g || !cfg || !run) return c.set(Status{GOPS_ERR_INVALID, "null argument"});
  if (g->impl.ctx != &c) return c.set(Status{GOPS_ERR_INVALID, "graph belongs to another context"});
  const Graph &gr = g->impl;
  if (gr.n > kNoAllocMaxNodes || gr.plan.n_hub_tasks > kNoAllocMaxHubTasks) {
    char msg[200];
    std::snprintf(msg, sizeof msg,
                  "gops_pagerank_run_noalloc: graph too large (n=%lld, hub tasks=%d; limits %lld nodes, "
                  "%lld hub tasks)",
                  (long long)gr.n, gr.plan.n_hub_tasks, (long long)kNoAllocMaxNodes,
                  (long long)kNoAllocMaxHubTasks);
    return c.set(Status{GOPS_ERR_INVALID, msg});
  }
  cudaError_t e = cudaSetDevice(c.device);
  if (e != cudaSuccess) return c.set(Status{GOPS_ERR_CUDA, cudaGetErrorString(e)});
  unsigned char *base = nullptr;
  Status st;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    st = scratch_address_locked(c.device, &base);
  }
  if (st.code != GOPS_OK) return c.set(st);
  Workspace ws = workspace_in(base);
  return c.set(solve_plain_in_workspace(&c, const_cast<Graph *>(&gr), cfg, ws, scores, run));
}
