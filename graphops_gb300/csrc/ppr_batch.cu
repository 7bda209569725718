// Batched personalized PageRank (K5): many seed sets per pass over the graph.
//
// Each seed set is one independent personalized_pagerank_run of the
// reference (src/ppr.rs:90-156) with personalization 1 on each seed node
// (repeats count), normalised as src/ppr.rs:104-109 does -- an empty set gives
// the uniform vector.  Sets run in waves of KT columns, KT = 32 * CPL with
// CPL (columns per lane) 1, 2 or 4.  Per wave the library keeps row-major
// (n+1) x KT blocks (relabelled node order) of the gathered step vector (FP32,
// plus a BF16 block of low words for the double-float phase), the
// double-float accumulator and the FP32 tail -- the residual form of the
// single solve (csrc/pagerank.cu), column by column:
//   r_1 = F(x_0) - x_0,  r_{k+1} = A r_k,  x_k = x_0 + sum r,  diff_k = ||r_k||_1
// with a double-float phase while some column's step norm is >= theta.
//
// Kernel layout: a warp owns a row and lane l owns columns l*CPL .. l*CPL +
// CPL - 1, so every gathered in-neighbour row is one coalesced KT * 4-byte
// read (128, 256 or 512 bytes in the FP32 phase), loaded as float / float2 /
// float4 per lane; the column indices of four edges come in one 16-byte
// broadcast load, and eight gathers per lane are in flight.  A wider k-tile
// reads the in-edge index stream once for more sets and moves more bytes per
// gather latency; the autotuner below picks it per graph.
//
// Canonical row sums.  A row's sum is defined independently of how the work
// is split: its in-edges form base blocks of kBase edges (from the row's
// first edge), each summed in edge order, and the block sums are added in
// block order.  Rows with more than `chunk` in-edges are split into chunk
// tasks (chunk a multiple of kBase) that write their blocks' sums, and the
// task that arrives last adds them in order.  So every k-tile and chunk size
// gives bit-identical results, and the autotuner's choice cannot change them.
//
// Per-column dangling and L1 sums are exact 64-bit fixed-point integers, so a
// column's result is independent of the others and of the schedule.  A
// column whose step norm fell below tol at step k-1 retires at step k: its
// values freeze (the reference returns that x) and it stops contributing;
// the wave ends when every column has retired or max_iterations is reached.
//
// Launch structure.  The kernels take no per-step or per-wave arguments: the
// step number comes from the wave record (k = k0 + j + 1 for the j-th step of
// a chunk; a one-thread kernel advances k0 after each chunk), the ping-pong
// buffers by its parity, and the per-wave constants from a device struct.  So
// a chunk of kChunkSteps steps is captured once as a CUDA graph and replayed
// for every chunk of every wave; the host polls a pinned copy of the wave
// record after each replay, with one chunk queued ahead.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <thread>
#include <vector>

#include "objects.cuh"
#include "primitives.cuh"

namespace gops {

constexpr int kMaxCPL = 4;
constexpr int kMaxKT = 32 * kMaxCPL;  // widest k-tile
constexpr int kBase = 256;            // edges per base block of a row sum
constexpr int kBThreads = 256;
constexpr int kBWarps = kBThreads / kWarp;
constexpr int kChunkSteps = 4;        // steps per launched (captured) chunk
constexpr double kBTheta = 1e-1;      // double-float phase while some column has ||r||_1 >= its theta
// judged warm starts (a finite r1_max): their first residual is already small
// (a learned start is typically 0.1-0.3), so the FP32 phase may begin at step
// 2; a column started from s (no judge, or a learned set over the push
// budget) keeps the cold threshold, whatever its wave
constexpr double kBThetaWarm = 5e-1;
// first step that skips the rows without in-edges (WaveScalars::skip_from):
// from a cold start the initialisation writes their zeros into gathered
// block 0 (and the accumulator and tail) and step 1 into block 1; after a
// caller's start vector step 1 writes its residual -x0, so steps 2 and 3
// write the zeros into both blocks first
constexpr int kSkipFromCold = 2;
constexpr int kSkipFromWarm = 4;

struct ColState {
  unsigned long long iterations;
  double diff_l1;
  int retired;
  int converged;
  int uniform;   // personalization is uniform (empty seed set)
  int rejected;  // warm start rejected after step 1 (its residual exceeded r1_max)
  double r1_max; // largest first-step residual accepted from a warm start
  double theta;  // double-float phase while this column's step norm >= theta
  int f32;       // in its FP32 phase (from the first step after its norm fell below theta)
  int pad;
};

struct WaveState {
  int done;
  int f32_phase;
  unsigned long long f32_from;
  unsigned long long steps;  // last step that did work
  unsigned long long k0;     // steps launched before the current chunk
};

// Per-call and per-wave values, read by the kernels from device memory.
struct WaveScalars {
  df d, omd, inv_n;
  float fx_scale;
  int ncols;
  double fx_inv;
  double tol;
  unsigned long long max_iter;
  int has_x0;
  int kt;  // columns of the wave's blocks (row stride)
  // From step skip_from on, rows without in-edges (rows [n_nz, n)) are
  // skipped but for the n_srow rows listed in srow (those of them that seed
  // a set of the wave): with no in-edge and no personalization their step
  // residual is exactly 0 (from step 1 from a cold start, from step 2 after
  // a caller's start vector), and everything the step would write for them
  // (tail, both gathered blocks, the double-float accumulator) already holds
  // that value once both blocks have been written with it.  A wave with a
  // uniform column (empty seed set) skips nothing.
  int skip_from;
  int n_srow;
};
struct WaveConst {
  WaveScalars s;
  int64_t xcol[kMaxKT], ocol[kMaxKT];  // set of each column: its row in x0 and in out
};

struct BatchState {
  int64_t n = 0;
  // tile configuration in use and the workspace's capacity
  int cpl = 0, chunk = 0;
  int kt_cap = 0;
  bool tuned = false;
  float tune_ms[3][2] = {};  // per (cpl 1/2/4, chunk 256/1024): cost per column-step, 0 = not tried
  float tune_l2 = 0.f;       // cost of the chosen tile with L2 eviction hints (0 = not tried)
  bool l2h = false;          // FP32 step with L2 eviction hints
  int l2_bytes = 0;          // the device's L2 size
  // chunk plan: rows [0, n_big) have more than `chunk` in-edges (rows are in
  // non-increasing in-degree); row h has tasks big_first[h]..big_first[h+1]-1
  // and base blocks blk_first[h]..blk_first[h+1]-1
  int32_t n_big = 0, n_big_tasks = 0, n_blocks = 0;
  int32_t *big_first = nullptr, *big_task_row = nullptr, *blk_first = nullptr;
  // wave workspace, kt_cap columns
  __nv_bfloat16 *glo[2] = {nullptr, nullptr};  // low words of the double-float gathered blocks (BF16)
  float *gf[2] = {nullptr, nullptr};           // gathered blocks: FP32, the double-float high words
  float2 *acc = nullptr;
  float *tail = nullptr;
  float2 *lpart = nullptr;   // base-block sums of chunked rows (n_blocks x kt_cap)
  unsigned *lcnt = nullptr;  // arrivals per chunked row
  long long *sums = nullptr; // 3 slots x kMaxKT x {dangling, l1, nonfinite, spare}
  ColState *cols = nullptr;  // kMaxKT
  WaveState *wave = nullptr;
  WaveConst *wc = nullptr;  // device
  int grid_df = 1, grid_f[2] = {1, 1};  // step kernel grids of the tile in use (FP32: without / with L2 hints)
  int32_t *prow = nullptr;    // n + 1
  int32_t *pslot = nullptr;   // seed entries of the wave: column slot
  float2 *pval = nullptr;     //   and normalised weight (double-float)
  int32_t *prows_sorted = nullptr;
  int32_t *srow = nullptr;    // the wave's seeded rows without in-edges (pcap entries)
  int64_t pcap = 0;
  int32_t n_nz = 0;           // rows with an in-edge: rows [0, n_nz) (in-degree order)
  float *x0 = nullptr;        // warm-start vectors of the wave (set-major, original order)
  float *out = nullptr;       // results of the wave (set-major, original order)
  int64_t x0_cols = 0, out_cols = 0;
  WaveState *hwave = nullptr;             // pinned: two polled copies of the wave record
  cudaEvent_t wev[2] = {nullptr, nullptr};
  std::vector<int32_t> inv_perm;  // host: original id -> relabelled row
  int32_t *d_inv_perm = nullptr;  // the same on the device
  // captured chunks: [0] double-float and FP32 launches, [1] FP32 only
  cudaGraphExec_t chunk_exec[2] = {nullptr, nullptr};
  int exec_cpl = 0, exec_chunk = 0, exec_l2h = -1;
  const void *exec_pslot = nullptr;
};

static void free_graphs(BatchState *b) {
  for (auto &e : b->chunk_exec)
    if (e) {
      cudaGraphExecDestroy(e);
      e = nullptr;
    }
  b->exec_cpl = 0;
}

static void free_plan(BatchState *b) {
  cudaFree(b->big_first); cudaFree(b->big_task_row); cudaFree(b->blk_first);
  cudaFree(b->lpart); cudaFree(b->lcnt);
  b->big_first = b->big_task_row = b->blk_first = nullptr;
  b->lpart = nullptr;
  b->lcnt = nullptr;
  b->n_big = b->n_big_tasks = b->n_blocks = 0;
  b->chunk = 0;
}

static void free_blocks(BatchState *b) {
  cudaFree(b->glo[0]); cudaFree(b->glo[1]); cudaFree(b->gf[0]); cudaFree(b->gf[1]);
  cudaFree(b->acc); cudaFree(b->tail);
  b->glo[0] = b->glo[1] = nullptr;
  b->gf[0] = b->gf[1] = nullptr;
  b->acc = nullptr;
  b->tail = nullptr;
  cudaFree(b->lpart);
  b->lpart = nullptr;
  b->kt_cap = 0;
}

void batch_free(Graph &g) {
  BatchState *b = g.batch;
  if (!b) return;
  free_graphs(b);
  free_plan(b);
  free_blocks(b);
  cudaFree(b->sums); cudaFree(b->cols); cudaFree(b->wave); cudaFree(b->wc); cudaFree(b->prow);
  cudaFree(b->pslot); cudaFree(b->pval); cudaFree(b->prows_sorted); cudaFree(b->srow); cudaFree(b->x0);
  cudaFree(b->out);
  cudaFree(b->d_inv_perm);
  if (b->hwave) cudaFreeHost(b->hwave);
  for (cudaEvent_t e : b->wev)
    if (e) cudaEventDestroy(e);
  delete b;
  g.batch = nullptr;
}

// Kernel arguments: fixed for a tile configuration (pointers only), so the
// launches of a chunk can be replayed from a captured graph.
struct StepParams {
  int64_t n;
  const int64_t *rp;
  const int32_t *col;
  const float *deg;
  const int32_t *perm;
  int32_t n_big, n_big_tasks, chunk;
  int32_t hot;  // rows [0, hot) of the gathered block kept in L2 (FP32 step with L2 hints)
  const int32_t *big_first, *big_task_row, *blk_first;
  const int32_t *prow, *pslot;
  const float2 *pval;
  int32_t n_nz;
  const int32_t *srow;
  __nv_bfloat16 *glo[2];
  float *gf[2];
  float2 *acc;
  float *tail;
  float2 *lpart;
  unsigned *lcnt;
  long long *sums;
  ColState *cols;
  WaveState *wave;
  const WaveConst *wc;
  int j;  // step offset within the chunk
};

namespace {

// ---------------------------------------------------------------------------
// lane values: CPL consecutive columns
// ---------------------------------------------------------------------------
template <int CPL>
struct FV {
  float v[CPL];
};
template <int CPL>
struct DV {
  df v[CPL];
};

template <int CPL>
__device__ __forceinline__ FV<CPL> ld_fv(const float *a) {
  FV<CPL> r;
  if constexpr (CPL == 1) {
    r.v[0] = __ldg(a);
  } else if constexpr (CPL == 2) {
    const float2 t = __ldg(reinterpret_cast<const float2 *>(a));
    r.v[0] = t.x; r.v[1] = t.y;
  } else {
    const float4 t = __ldg(reinterpret_cast<const float4 *>(a));
    r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
  }
  return r;
}

template <int CPL>
__device__ __forceinline__ void st_fv(float *a, const FV<CPL> &r) {
  if constexpr (CPL == 1) {
    *a = r.v[0];
  } else if constexpr (CPL == 2) {
    *reinterpret_cast<float2 *>(a) = make_float2(r.v[0], r.v[1]);
  } else {
    *reinterpret_cast<float4 *>(a) = make_float4(r.v[0], r.v[1], r.v[2], r.v[3]);
  }
}

// L2 eviction priorities (createpolicy / cache_hint): evict_last for the
// rows of the gathered block that most in-edges read (the first rows after
// the in-degree relabelling), evict_first for everything streamed once.
__device__ __forceinline__ uint64_t pol_first() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t pol_last() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}

template <int CPL>
__device__ __forceinline__ FV<CPL> ld_fv_pol(const float *a, uint64_t pol) {
  FV<CPL> r;
  if constexpr (CPL == 1) {
    asm volatile("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(r.v[0]) : "l"(a), "l"(pol));
  } else if constexpr (CPL == 2) {
    asm volatile("ld.global.nc.L2::cache_hint.v2.f32 {%0,%1}, [%2], %3;" : "=f"(r.v[0]), "=f"(r.v[1]) : "l"(a), "l"(pol));
  } else {
    asm volatile("ld.global.nc.L2::cache_hint.v4.f32 {%0,%1,%2,%3}, [%4], %5;"
                 : "=f"(r.v[0]), "=f"(r.v[1]), "=f"(r.v[2]), "=f"(r.v[3]) : "l"(a), "l"(pol));
  }
  return r;
}

template <int CPL>
__device__ __forceinline__ void st_fv_pol(float *a, const FV<CPL> &r, uint64_t pol) {
  if constexpr (CPL == 1) {
    asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(a), "f"(r.v[0]), "l"(pol) : "memory");
  } else if constexpr (CPL == 2) {
    asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1,%2}, %3;" ::"l"(a), "f"(r.v[0]), "f"(r.v[1]), "l"(pol)
                 : "memory");
  } else {
    asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1,%2,%3,%4}, %5;" ::"l"(a), "f"(r.v[0]), "f"(r.v[1]),
                 "f"(r.v[2]), "f"(r.v[3]), "l"(pol) : "memory");
  }
}

__device__ __forceinline__ int4 ld_i4_pol(const int32_t *a, uint64_t pol) {
  int4 v;
  asm volatile("ld.global.nc.L2::cache_hint.v4.s32 {%0,%1,%2,%3}, [%4], %5;"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(a), "l"(pol));
  return v;
}

// CPL double-float values stored as CPL float2 (hi, lo)
template <int CPL>
__device__ __forceinline__ DV<CPL> ld_dv(const float2 *a, bool cached) {
  DV<CPL> r;
  if constexpr (CPL == 1) {
    const float2 t = cached ? __ldg(a) : *a;
    r.v[0] = {t.x, t.y};
  } else {
#pragma unroll
    for (int q = 0; q < CPL / 2; ++q) {
      const float4 t = cached ? __ldg(reinterpret_cast<const float4 *>(a) + q) : reinterpret_cast<const float4 *>(a)[q];
      r.v[2 * q] = {t.x, t.y};
      r.v[2 * q + 1] = {t.z, t.w};
    }
  }
  return r;
}

template <int CPL>
__device__ __forceinline__ void st_dv(float2 *a, const DV<CPL> &r) {
  if constexpr (CPL == 1) {
    *a = make_float2(r.v[0].hi, r.v[0].lo);
  } else {
#pragma unroll
    for (int q = 0; q < CPL / 2; ++q)
      reinterpret_cast<float4 *>(a)[q] = make_float4(r.v[2 * q].hi, r.v[2 * q].lo, r.v[2 * q + 1].hi, r.v[2 * q + 1].lo);
  }
}

// Low words of CPL double-float entries, kept as BF16 (the high words are
// the FP32 block): loaded as one 8-, 4- or 2-byte read, widened exactly.
template <int CPL>
__device__ __forceinline__ void ld_lo(const __nv_bfloat16 *a, float (&lo)[CPL]) {
  const unsigned short *h = reinterpret_cast<const unsigned short *>(a);
  if constexpr (CPL == 1) {
    lo[0] = __uint_as_float((uint32_t)__ldg(h) << 16);
  } else if constexpr (CPL == 2) {
    const uint32_t t = __ldg(reinterpret_cast<const unsigned int *>(h));
    lo[0] = __uint_as_float(t << 16);
    lo[1] = __uint_as_float(t & 0xFFFF0000u);
  } else {
    const uint2 t = __ldg(reinterpret_cast<const uint2 *>(h));
    lo[0] = __uint_as_float(t.x << 16);
    lo[1] = __uint_as_float(t.x & 0xFFFF0000u);
    lo[2] = __uint_as_float(t.y << 16);
    lo[3] = __uint_as_float(t.y & 0xFFFF0000u);
  }
}

__device__ __forceinline__ uint32_t bf16_bits(float v) {
  const __nv_bfloat16 b = __float2bfloat16_rn(v);
  return (uint32_t)*reinterpret_cast<const unsigned short *>(&b);
}

template <int CPL>
__device__ __forceinline__ void st_lo(__nv_bfloat16 *a, const DV<CPL> &r) {
  unsigned short *h = reinterpret_cast<unsigned short *>(a);
  if constexpr (CPL == 1) {
    *h = (unsigned short)bf16_bits(r.v[0].lo);
  } else if constexpr (CPL == 2) {
    *reinterpret_cast<unsigned int *>(h) = bf16_bits(r.v[0].lo) | (bf16_bits(r.v[1].lo) << 16);
  } else {
    *reinterpret_cast<uint2 *>(h) = make_uint2(bf16_bits(r.v[0].lo) | (bf16_bits(r.v[1].lo) << 16),
                                               bf16_bits(r.v[2].lo) | (bf16_bits(r.v[3].lo) << 16));
  }
}

// FP32 step of one column (shared by both kernels, with explicit roundings
// so that the two compute the same bits): r = d (s + dsum * red).
__device__ __forceinline__ float f32_step(float s, float dsum, float red, float d) {
  return __fmul_rn(d, __fmaf_rn(dsum, red, s));
}

// ---------------------------------------------------------------------------
// The FP32 step (every active column in its FP32 phase): gathers KT * 4-byte
// rows of the FP32 block.
// ---------------------------------------------------------------------------
template <int CPL>
__device__ __forceinline__ void f32_add(FV<CPL> &s, const FV<CPL> &g) {
#pragma unroll
  for (int q = 0; q < CPL; ++q) s.v[q] += g.v[q];
}

template <int CPL>
__device__ __forceinline__ FV<CPL> f32_zero() {
  FV<CPL> r;
#pragma unroll
  for (int q = 0; q < CPL; ++q) r.v[q] = 0.0f;
  return r;
}

// Sum over edges [eb, ee) of one base block, in edge order.  Rows are
// padded to multiples of 4 edges and start 16-byte aligned; padding edges
// point at row n, whose gathered entries are 0.
// With L2H the column indices stream evict-first and the gathers of rows
// below p.hot are marked evict-last.
template <int CPL, bool L2H>
__device__ __forceinline__ FV<CPL> gather_fv(const StepParams &p, const float *gb, int32_t u, int kt) {
  if constexpr (L2H) return ld_fv_pol<CPL>(gb + (int64_t)u * kt, u < p.hot ? pol_last() : pol_first());
  else return ld_fv<CPL>(gb + (int64_t)u * kt);
}

template <bool L2H>
__device__ __forceinline__ int4 col_quad(const StepParams &p, int e) {
  if constexpr (L2H) return ld_i4_pol(p.col + e, pol_first());
  else return __ldg(reinterpret_cast<const int4 *>(p.col + e));
}

template <int CPL, bool L2H>
__device__ __forceinline__ FV<CPL> f32_block(const StepParams &p, int in, int kt, int eb, int ee, int lane) {
  constexpr int U = 8;  // gathers in flight per lane
  const float *gb = p.gf[in] + lane * CPL;
  FV<CPL> s = f32_zero<CPL>();
  int e = eb;
  for (; e + U <= ee; e += U) {
    const int4 a = col_quad<L2H>(p, e);
    const int4 b = col_quad<L2H>(p, e + 4);
    const int32_t u[U] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    FV<CPL> g[U];
#pragma unroll
    for (int q = 0; q < U; ++q) g[q] = gather_fv<CPL, L2H>(p, gb, u[q], kt);
#pragma unroll
    for (int q = 0; q < U; ++q) f32_add(s, g[q]);
  }
  if (e < ee) {
    const int4 a = col_quad<L2H>(p, e);
    const int32_t u[4] = {a.x, a.y, a.z, a.w};
    FV<CPL> g[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) g[q] = gather_fv<CPL, L2H>(p, gb, u[q], kt);
#pragma unroll
    for (int q = 0; q < 4; ++q) f32_add(s, g[q]);
  }
  return s;
}

// ---------------------------------------------------------------------------
// The mixed step (some active column still in its double-float phase).
// Every lane gathers its double-float entries: the high words from the FP32
// block and the low words from the BF16 low-word block (6 bytes per entry;
// a stored value keeps 24 + 8 significant bits, far more than the FP32
// phase's sums, while the gathers move 3/4 of full double-float's bytes).
// A column in its double-float phase adds them in double-float arithmetic; a
// column already in its FP32 phase adds only the hi words in FP32 (its sum
// kept in the hi word), which is exactly what the FP32 step computes from the
// FP32 block (the double-float step writes hi there).  So every column's
// result depends on its own history alone: not on the sets that share its
// wave, nor on the k-tile.
// ---------------------------------------------------------------------------
template <int CPL>
struct MixSum {
  DV<CPL> d;  // double-float sums (columns in the double-float phase)
  FV<CPL> f;  // FP32 sums of the hi words (columns in the FP32 phase)
};

template <int CPL>
__device__ __forceinline__ MixSum<CPL> mix_zero() {
  MixSum<CPL> r;
#pragma unroll
  for (int q = 0; q < CPL; ++q) {
    r.d.v[q] = {0.0f, 0.0f};
    r.f.v[q] = 0.0f;
  }
  return r;
}

// One gathered entry into a base block's sums: the high words with an exact
// two-sum (Knuth), its error and the entry's low word into an FP32 low word
// that is renormalised once per base block (mix_normalize), 8 instead of
// 11 FP32 operations per double-float column; the low sum of a 256-edge
// block keeps the result to about 2^-32 of its largest term, the precision
// of the stored (BF16) low words themselves.  WANT_F: some column of the
// wave is in its FP32 phase and needs the FP32 sum of the high words.
template <int CPL, bool WANT_F>
__device__ __forceinline__ void mix_add(MixSum<CPL> &s, const DV<CPL> &g) {
#pragma unroll
  for (int q = 0; q < CPL; ++q) {
    const df t = two_sum(s.d.v[q].hi, g.v[q].hi);
    s.d.v[q] = {t.hi, __fadd_rn(s.d.v[q].lo, __fadd_rn(t.lo, g.v[q].lo))};
    if constexpr (WANT_F) s.f.v[q] += g.v[q].hi;
  }
}

// the base block's double-float sums back to (hi, lo) with |lo| <= ulp(hi)/2
// (a full two-sum: the high sum may have cancelled below the low one)
template <int CPL>
__device__ __forceinline__ void mix_normalize(MixSum<CPL> &s) {
#pragma unroll
  for (int q = 0; q < CPL; ++q) s.d.v[q] = two_sum(s.d.v[q].hi, s.d.v[q].lo);
}

template <int CPL>
__device__ __forceinline__ void mix_add(MixSum<CPL> &s, const MixSum<CPL> &t) {
#pragma unroll
  for (int q = 0; q < CPL; ++q) {
    s.d.v[q] = df_add(s.d.v[q], t.d.v[q]);
    s.f.v[q] += t.f.v[q];
  }
}

template <int CPL>
__device__ __forceinline__ DV<CPL> gather_dv(const float *ghi, const __nv_bfloat16 *glo, int64_t off) {
  const FV<CPL> h = ld_fv<CPL>(ghi + off);
  float lo[CPL];
  ld_lo<CPL>(glo + off, lo);
  DV<CPL> r;
#pragma unroll
  for (int q = 0; q < CPL; ++q) r.v[q] = {h.v[q], lo[q]};
  return r;
}

template <int CPL, bool WANT_F>
__device__ __forceinline__ MixSum<CPL> mix_block(const StepParams &p, int in, int kt, int eb, int ee, int lane) {
  constexpr int U = CPL == 4 ? 4 : 8;
  const float *ghi = p.gf[in] + lane * CPL;
  const __nv_bfloat16 *glo = p.glo[in] + lane * CPL;
  MixSum<CPL> s = mix_zero<CPL>();
  for (int e = eb; e < ee; e += U) {  // ee - eb is a multiple of 4
    int32_t u[U];
    const int4 a = __ldg(reinterpret_cast<const int4 *>(p.col + e));
    u[0] = a.x; u[1] = a.y; u[2] = a.z; u[3] = a.w;
    bool ok2 = true;
    if constexpr (U == 8) {
      ok2 = e + 4 < ee;
      const int4 b = ok2 ? __ldg(reinterpret_cast<const int4 *>(p.col + e + 4)) : make_int4(0, 0, 0, 0);
      u[4] = b.x; u[5] = b.y; u[6] = b.z; u[7] = b.w;
    }
    DV<CPL> g[U];
#pragma unroll
    for (int q = 0; q < U; ++q)
      if (q < 4 || ok2) g[q] = gather_dv<CPL>(ghi, glo, (int64_t)u[q] * kt);
#pragma unroll
    for (int q = 0; q < U; ++q)
      if (q < 4 || ok2) mix_add<CPL, WANT_F>(s, g[q]);
  }
  mix_normalize<CPL>(s);
  return s;
}

struct Lane {
  // per column of this lane
  bool act[kMaxCPL];
  bool f32[kMaxCPL];  // in its FP32 phase
  bool uni[kMaxCPL];
  df dsum[kMaxCPL];
  bool any;        // some column active
  unsigned fmask;  // bit q: column q active and in its FP32 phase
};

// A lane's exact fixed-point partial sums (L1 norm and dangling mass per
// column, and a nonfinite bit per column), kept in its warp's shared-memory
// slots rather than in registers; block_sums adds them up per column.
template <int CPL>
struct LaneAcc {
  long long *l1, *dang;
  int *bad;
  __device__ LaneAcc(long long *l, long long *d, int *b) : l1(l), dang(d), bad(b) {
#pragma unroll
    for (int q = 0; q < CPL; ++q) l1[q] = dang[q] = 0;
    *bad = 0;
  }
};

// Per-(row, lane) epilogue inputs, loaded before the row's gathers.
template <int CPL>
struct BIn {
  df red[CPL];
  FV<CPL> tail;
  DV<CPL> acc;  // double-float lanes only
  float deg;
};

template <int CPL, bool L2H = false>
__device__ __forceinline__ BIn<CPL> b_in(const StepParams &p, const WaveScalars &wc, int64_t v, int lane,
                                         const Lane &ln, bool want_acc, bool want_tail) {
  BIn<CPL> in;
#pragma unroll
  for (int q = 0; q < CPL; ++q) in.red[q] = ln.uni[q] ? wc.inv_n : df{0.0f, 0.0f};
  const int pb = __ldg(&p.prow[v]), pe = __ldg(&p.prow[v + 1]);
  for (int e = pb; e < pe; ++e) {
    const int q = __ldg(&p.pslot[e]) - lane * CPL;
    if (q >= 0 && q < CPL) {
      const float2 w = __ldg(&p.pval[e]);
#pragma unroll
      for (int qq = 0; qq < CPL; ++qq)
        if (qq == q) in.red[qq] = {w.x, w.y};
    }
  }
  in.deg = __ldg(&p.deg[v]);
  const int64_t i = v * wc.kt + lane * CPL;
  if (want_tail) {
    if constexpr (L2H) in.tail = ld_fv_pol<CPL>(p.tail + i, pol_first());
    else in.tail = ld_fv<CPL>(p.tail + i);
  }
  if (want_acc) in.acc = ld_dv<CPL>(p.acc + i, false);
  return in;
}

// FP32 step epilogue: every active column of the lane in its FP32 phase.
template <int CPL, bool L2H = false>
__device__ __forceinline__ void f32_epilogue(const StepParams &p, const WaveScalars &wc, int64_t v, const FV<CPL> &s,
                                             const BIn<CPL> &in, const Lane &ln, int out, LaneAcc<CPL> &a, int lane) {
  const int64_t i = v * wc.kt + lane * CPL;
  const float dg = in.deg;
  FV<CPL> tn, gh;
#pragma unroll
  for (int q = 0; q < CPL; ++q) {
    const float r = ln.act[q] ? f32_step(s.v[q], ln.dsum[q].hi, in.red[q].hi, wc.d.hi) : 0.0f;
    tn.v[q] = in.tail.v[q] + r;
    a.l1[q] += fx_of(fabsf(r), wc.fx_scale);
    *a.bad |= (!isfinite(r)) << q;
    if (dg == 0.0f) a.dang[q] += fx_of(r, wc.fx_scale);
    gh.v[q] = dg > 0.0f ? __fdiv_rn(r, dg) : 0.0f;
  }
  if constexpr (L2H) {
    st_fv_pol<CPL>(p.tail + i, tn, pol_first());
    st_fv_pol<CPL>(p.gf[out] + i, gh, v < p.hot ? pol_last() : pol_first());
  } else {
    st_fv<CPL>(p.tail + i, tn);
    st_fv<CPL>(p.gf[out] + i, gh);
  }
}

// Mixed step epilogue: a column in its double-float phase takes the
// double-float step on its double-float sum (x in acc), one in its FP32
// phase the FP32 step on the hi word of its sum (x in tail), exactly as
// f32_epilogue computes it.  The tail is read and written only by lanes with
// such a column.
template <int CPL>
__device__ __forceinline__ void mix_epilogue(const StepParams &p, const WaveScalars &wc, int64_t v, const MixSum<CPL> &s,
                                             const BIn<CPL> &in, const Lane &ln, int out, unsigned long long k,
                                             LaneAcc<CPL> &a, int lane) {
  const int64_t i = v * wc.kt + lane * CPL;
  const float dg = in.deg;
  DV<CPL> an, g;
  FV<CPL> tn, gh;
#pragma unroll
  for (int q = 0; q < CPL; ++q) {
    const df red = in.red[q];
    an.v[q] = in.acc.v[q];
    tn.v[q] = ln.fmask ? in.tail.v[q] : 0.0f;
    if (ln.act[q] && ln.f32[q]) {
      const float r = f32_step(s.f.v[q], ln.dsum[q].hi, red.hi, wc.d.hi);
      tn.v[q] = in.tail.v[q] + r;
      a.l1[q] += fx_of(fabsf(r), wc.fx_scale);
      *a.bad |= (!isfinite(r)) << q;
      if (dg == 0.0f) a.dang[q] += fx_of(r, wc.fx_scale);
      gh.v[q] = dg > 0.0f ? __fdiv_rn(r, dg) : 0.0f;
      g.v[q] = {gh.v[q], 0.0f};
    } else if (ln.act[q]) {
      const df ao = in.acc.v[q];
      df r = df_mul(wc.d, df_add(s.d.v[q], df_mul(ln.dsum[q], red)));
      if (k == 1) r = df_add(df_add(df_mul(wc.omd, red), r), df_neg(ao));  // F(x_0) - x_0
      an.v[q] = df_add(ao, r);
      const df ar = r.hi < 0.0f ? df_neg(r) : r;
      a.l1[q] += fx_of(ar.hi, wc.fx_scale) + fx_of(ar.lo, wc.fx_scale);
      *a.bad |= (!isfinite(r.hi)) << q;
      if (dg == 0.0f) a.dang[q] += fx_of(r.hi, wc.fx_scale) + fx_of(r.lo, wc.fx_scale);
      g.v[q] = dg > 0.0f ? df_div_f(r, dg) : df{0.0f, 0.0f};
      gh.v[q] = g.v[q].hi;
    } else {
      g.v[q] = {0.0f, 0.0f};
      gh.v[q] = 0.0f;
    }
  }
  st_dv<CPL>(p.acc + i, an);
  if (ln.fmask) st_fv<CPL>(p.tail + i, tn);
  st_lo<CPL>(p.glo[out] + i, g);
  st_fv<CPL>(p.gf[out] + i, gh);
}

// Per-column view of step k: which columns are still active, which are in
// their FP32 phase (sticky: from the first step after their step norm fell
// below their theta), their dangling sums, and whether this kernel (the
// mixed step: WANT_MIX, or the FP32 step) is the one to run.  Returns false
// when the block should exit.  Every warp evaluates it identically.
template <bool WANT_MIX, int CPL>
__device__ bool batch_prologue(const StepParams &p, const WaveScalars &wc, unsigned long long k, int lane, Lane *ln) {
  if (*(volatile int *)&p.wave->done) return false;
  const int prev = (int)((k - 1) % 3);
  bool lane_act = false, lane_df = false;
  unsigned fmask = 0;
#pragma unroll
  for (int q = 0; q < CPL; ++q) {
    const int c = lane * CPL + q;
    const bool col_ok = c < wc.ncols;
    const int retired0 = col_ok ? *(volatile int *)&p.cols[c].retired : 1;
    double diff = INFINITY;
    if (k > 1) {
      const long long raw = *(volatile long long *)&p.sums[(prev * kMaxKT + c) * 4 + 1];
      const long long badc = *(volatile long long *)&p.sums[(prev * kMaxKT + c) * 4 + 2];
      diff = badc ? NAN : (double)raw * wc.fx_inv;
    }
    // a warm start is judged by its first residual: one that does not drop
    // below the cold start's (or is not finite) retires the column, and the
    // caller solves that set again from the personalization vector
    const bool rej = !retired0 && k == 2 && wc.has_x0 && !(diff <= p.cols[c].r1_max);
    const bool conv = !retired0 && !rej && k > 1 && diff < wc.tol;
    const bool cap = !retired0 && !rej && !conv && k - 1 >= wc.max_iter;
    const bool act = !retired0 && !rej && !conv && !cap;
    const bool f32 = act && k > 1 && (*(volatile int *)&p.cols[c].f32 || diff < p.cols[c].theta);
    if (blockIdx.x == 0 && threadIdx.x < 32) {
      if (conv || cap || rej) {
        p.cols[c].retired = 1;
        p.cols[c].converged = conv ? 1 : 0;
        p.cols[c].rejected = rej ? 1 : 0;
        p.cols[c].iterations = k - 1;
        p.cols[c].diff_l1 = diff;
      }
      if (f32) p.cols[c].f32 = 1;
    }
    ln->act[q] = act;
    ln->f32[q] = f32;
    ln->uni[q] = col_ok && p.cols[c].uniform;
    lane_act |= act;
    lane_df |= act && !f32;
    fmask |= (act && f32 ? 1u : 0u) << q;
  }
  ln->any = lane_act;
  ln->fmask = fmask;
  if (!__any_sync(0xffffffffu, lane_act)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) p.wave->done = 1;
    return false;
  }
  const bool all_f32 = k > 1 && (*(volatile int *)&p.wave->f32_phase || !__any_sync(0xffffffffu, lane_df));
  if (all_f32 == WANT_MIX) return false;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    p.wave->f32_phase = all_f32 ? 1 : 0;
    if (all_f32 && p.wave->f32_from == 0) p.wave->f32_from = k;
    p.wave->steps = k;
  }
  if (blockIdx.x == 0 && threadIdx.x < kMaxKT) {
    const int nxt = (int)((k + 1) % 3);
    for (int i = 0; i < 4; ++i) p.sums[(nxt * kMaxKT + threadIdx.x) * 4 + i] = 0;
  }
#pragma unroll
  for (int q = 0; q < CPL; ++q) {
    const long long draw = *(volatile long long *)&p.sums[(prev * kMaxKT + lane * CPL + q) * 4 + 0];
    ln->dsum[q] = df_from_double((double)draw * wc.fx_inv);
  }
  return true;
}

// The block's per-column fixed-point sums -> one atomic per column.
template <int CPL>
__device__ __forceinline__ void block_sums(const StepParams &p, int kt, unsigned long long k,
                                           long long (*bl1)[kMaxKT], long long (*bdg)[kMaxKT], int (*bbad)[32]) {
  __syncthreads();
  if (threadIdx.x < kt) {
    const int c = threadIdx.x;
    long long t1 = 0, t2 = 0;
    int tb = 0;
    for (int w = 0; w < kBWarps; ++w) {
      t1 += bl1[w][c];
      t2 += bdg[w][c];
      tb |= (bbad[w][c / CPL] >> (c % CPL)) & 1;
    }
    const int cur = (int)(k % 3);
    long long *sl = &p.sums[(cur * kMaxKT + c) * 4];
    if (t1) atomicAdd((unsigned long long *)&sl[1], (unsigned long long)t1);
    if (t2) atomicAdd((unsigned long long *)&sl[0], (unsigned long long)t2);
    if (tb) atomicAdd((unsigned long long *)&sl[2], 1ull);
  }
}

// Chunk task t of a row with more than `chunk` in-edges: its row h, the
// row's tasks and base blocks, and the task's edge range [cs, ce).  The
// task writes the sums of its base blocks to lpart; chunk_arrive returns
// true for the task that arrives last, which adds the row's blocks in order
// and runs the epilogue.
__device__ __forceinline__ void chunk_row(const StepParams &p, int t, int *h, int *first, int *nch, int *b0, int *nb,
                                          int *cs, int *ce, int *rb) {
  *h = __ldg(&p.big_task_row[t]);
  *first = __ldg(&p.big_first[*h]);
  *nch = __ldg(&p.big_first[*h + 1]) - *first;
  *b0 = __ldg(&p.blk_first[*h]);
  *nb = __ldg(&p.blk_first[*h + 1]) - *b0;
  *rb = (int)__ldg(&p.rp[*h]);
  const int re = (int)__ldg(&p.rp[*h + 1]);
  *cs = *rb + (t - *first) * p.chunk;
  *ce = min(re, *cs + p.chunk);
}

__device__ __forceinline__ bool chunk_arrive(const StepParams &p, int h, int nch, int lane) {
  __threadfence();
  __syncwarp();
  unsigned tk = 0;
  if (lane == 0) tk = atomicAdd(&p.lcnt[h], 1u);
  tk = __shfl_sync(0xffffffffu, tk, 0);
  if (tk != (unsigned)(nch - 1)) return false;
  __threadfence();
  if (lane == 0) p.lcnt[h] = 0;
  return true;
}

template <int CPL, bool L2H>
__global__ void __launch_bounds__(kBThreads) spmm_f32(StepParams p) {
  __shared__ long long bl1[kBWarps][kMaxKT], bdg[kBWarps][kMaxKT];
  __shared__ int bbad[kBWarps][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const WaveScalars wc = p.wc->s;
  const unsigned long long k = *(volatile unsigned long long *)&p.wave->k0 + (unsigned long long)p.j + 1ull;
  Lane ln;
  if (!batch_prologue<false, CPL>(p, wc, k, lane, &ln)) return;
  const int in = (int)((k - 1) & 1), out = (int)(k & 1);
  const int kt = wc.kt;
  LaneAcc<CPL> a(&bl1[wid][lane * CPL], &bdg[wid][lane * CPL], &bbad[wid][lane]);
  const int64_t nwarps = (int64_t)gridDim.x * kBWarps;
  const bool skip = k >= (unsigned long long)wc.skip_from;
  const int64_t nreg = (skip ? (int64_t)p.n_nz : p.n) - p.n_big;  // regular rows taken in order
  const int64_t nwt = p.n_big_tasks + nreg + (skip ? wc.n_srow : 0);
  for (int64_t w = (int64_t)blockIdx.x * kBWarps + wid; w < nwt; w += nwarps) {
    if (w < p.n_big_tasks) {
      int h, first, nch, b0, nb, cs, ce, rb;
      chunk_row(p, (int)w, &h, &first, &nch, &b0, &nb, &cs, &ce, &rb);
      // a lane whose columns have all retired gathers nothing
      if (ln.any)
        for (int b = cs; b < ce; b += kBase) {
          const FV<CPL> s = f32_block<CPL, L2H>(p, in, kt, b, min(ce, b + kBase), lane);
          DV<CPL> pk;
#pragma unroll
          for (int q = 0; q < CPL; ++q) pk.v[q] = {s.v[q], 0.0f};
          st_dv<CPL>(p.lpart + (int64_t)(b0 + (b - rb) / kBase) * kt + lane * CPL, pk);
        }
      if (chunk_arrive(p, h, nch, lane) && ln.any) {
        const BIn<CPL> bi = b_in<CPL, L2H>(p, wc, h, lane, ln, false, true);
        FV<CPL> all = f32_zero<CPL>();
        for (int q = 0; q < nb; ++q) {
          const DV<CPL> d = ld_dv<CPL>(p.lpart + (int64_t)(b0 + q) * kt + lane * CPL, false);
#pragma unroll
          for (int j = 0; j < CPL; ++j) all.v[j] = q == 0 ? d.v[j].hi : all.v[j] + d.v[j].hi;
        }
        f32_epilogue<CPL, L2H>(p, wc, h, all, bi, ln, out, a, lane);
      }
    } else if (ln.any) {
      const int64_t r = w - p.n_big_tasks;
      const int64_t v = r < nreg ? p.n_big + r : (int64_t)__ldg(&p.srow[r - nreg]);
      const BIn<CPL> bi = b_in<CPL, L2H>(p, wc, v, lane, ln, false, true);
      const int eb = (int)__ldg(&p.rp[v]), ee = (int)__ldg(&p.rp[v + 1]);
      // canonical row sum: base blocks from eb, added in order
      FV<CPL> tot = f32_block<CPL, L2H>(p, in, kt, eb, min(ee, eb + kBase), lane);
      for (int b = eb + kBase; b < ee; b += kBase)
        f32_add(tot, f32_block<CPL, L2H>(p, in, kt, b, min(ee, b + kBase), lane));
      f32_epilogue<CPL, L2H>(p, wc, v, tot, bi, ln, out, a, lane);
    }
  }
  block_sums<CPL>(p, kt, k, bl1, bdg, bbad);
}

template <int CPL>
__global__ void __launch_bounds__(kBThreads, 2) spmm_mixed(StepParams p) {
  __shared__ long long bl1[kBWarps][kMaxKT], bdg[kBWarps][kMaxKT];
  __shared__ int bbad[kBWarps][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const WaveScalars wc = p.wc->s;
  const unsigned long long k = *(volatile unsigned long long *)&p.wave->k0 + (unsigned long long)p.j + 1ull;
  Lane ln;
  if (!batch_prologue<true, CPL>(p, wc, k, lane, &ln)) return;
  const int in = (int)((k - 1) & 1), out = (int)(k & 1);
  const int kt = wc.kt;
  LaneAcc<CPL> a(&bl1[wid][lane * CPL], &bdg[wid][lane * CPL], &bbad[wid][lane]);
  const int64_t nwarps = (int64_t)gridDim.x * kBWarps;
  const bool skip = k >= (unsigned long long)wc.skip_from;
  const int64_t nreg = (skip ? (int64_t)p.n_nz : p.n) - p.n_big;  // regular rows taken in order
  const int64_t nwt = p.n_big_tasks + nreg + (skip ? wc.n_srow : 0);
  // At 4 columns per lane the FP32 sums of the high words are kept only when
  // some column is in its FP32 phase (the same for every warp: they read the
  // same column records); narrower tiles keep one variant, within their
  // register budget.
  const bool want_f = __any_sync(0xffffffffu, ln.fmask != 0u);
  auto block_sum = [&](int b0_, int b1_) {
    if constexpr (CPL == 4)
      if (!want_f) return mix_block<CPL, false>(p, in, kt, b0_, b1_, lane);
    return mix_block<CPL, true>(p, in, kt, b0_, b1_, lane);
  };
  for (int64_t w = (int64_t)blockIdx.x * kBWarps + wid; w < nwt; w += nwarps) {
    if (w < p.n_big_tasks) {
      int h, first, nch, b0, nb, cs, ce, rb;
      chunk_row(p, (int)w, &h, &first, &nch, &b0, &nb, &cs, &ce, &rb);
      if (ln.any)
        for (int b = cs; b < ce; b += kBase) {
          // per column: the double-float sum, or the FP32 sum as (s, 0)
          const MixSum<CPL> s = block_sum(b, min(ce, b + kBase));
          DV<CPL> pk;
#pragma unroll
          for (int q = 0; q < CPL; ++q) pk.v[q] = ((ln.fmask >> q) & 1u) ? df{s.f.v[q], 0.0f} : s.d.v[q];
          st_dv<CPL>(p.lpart + (int64_t)(b0 + (b - rb) / kBase) * kt + lane * CPL, pk);
        }
      if (chunk_arrive(p, h, nch, lane) && ln.any) {
        const BIn<CPL> bi = b_in<CPL>(p, wc, h, lane, ln, true, ln.fmask != 0);
        MixSum<CPL> all = mix_zero<CPL>();
        for (int q = 0; q < nb; ++q) {
          const DV<CPL> d = ld_dv<CPL>(p.lpart + (int64_t)(b0 + q) * kt + lane * CPL, false);
#pragma unroll
          for (int j = 0; j < CPL; ++j) {
            all.d.v[j] = q == 0 ? d.v[j] : df_add(all.d.v[j], d.v[j]);
            all.f.v[j] = q == 0 ? d.v[j].hi : all.f.v[j] + d.v[j].hi;
          }
        }
        mix_epilogue<CPL>(p, wc, h, all, bi, ln, out, k, a, lane);
      }
    } else if (ln.any) {
      const int64_t r = w - p.n_big_tasks;
      const int64_t v = r < nreg ? p.n_big + r : (int64_t)__ldg(&p.srow[r - nreg]);
      const BIn<CPL> bi = b_in<CPL>(p, wc, v, lane, ln, true, ln.fmask != 0);
      const int eb = (int)__ldg(&p.rp[v]), ee = (int)__ldg(&p.rp[v + 1]);
      MixSum<CPL> tot = block_sum(eb, min(ee, eb + kBase));
      for (int b = eb + kBase; b < ee; b += kBase) mix_add<CPL>(tot, block_sum(b, min(ee, b + kBase)));
      mix_epilogue<CPL>(p, wc, v, tot, bi, ln, out, k, a, lane);
    }
  }
  block_sums<CPL>(p, kt, k, bl1, bdg, bbad);
}

// the wave record's step counter after a chunk
__global__ void advance_kernel(WaveState *wave) { wave->k0 += kChunkSteps; }

// personalization entry of (row v, column c), double-float
__device__ __forceinline__ df red_of(const StepParams &p, const WaveScalars &wc, int64_t v, int c, bool uniform) {
  if (uniform) return wc.inv_n;
  df red = {0.0f, 0.0f};
  const int pb = __ldg(&p.prow[v]), pe = __ldg(&p.prow[v + 1]);
  for (int e = pb; e < pe; ++e)
    if (__ldg(&p.pslot[e]) == c) {
      const float2 w = __ldg(&p.pval[e]);
      red = {w.x, w.y};
    }
  return red;
}

// x_0 = p, acc = x_0, tail = 0, gathered blocks for step 1, per-column
// dangling sums of x_0; zero padding row n of both gathered blocks.  One
// thread per (row, column) entry, columns fastest.
__global__ void __launch_bounds__(kBThreads) batch_init(StepParams p) {
  __shared__ long long bdg[kMaxKT];
  const WaveScalars wc = p.wc->s;
  const int kt = wc.kt;
  for (int c = threadIdx.x; c < kt; c += blockDim.x) bdg[c] = 0;
  __syncthreads();
  const int64_t total = (p.n + 1) * kt;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = i / kt;
    const int c = (int)(i - v * kt);
    if (v == p.n) {
      p.glo[0][i] = p.glo[1][i] = __float2bfloat16_rn(0.f);
      p.gf[0][i] = p.gf[1][i] = 0.f;
      continue;
    }
    const bool col_ok = c < wc.ncols;
    const df x0 = col_ok ? red_of(p, wc, v, c, p.cols[c].uniform != 0) : df{0.f, 0.f};
    const float dg = p.deg[v];
    p.acc[i] = make_float2(x0.hi, x0.lo);
    p.tail[i] = 0.f;
    const df g = dg > 0.f ? df_div_f(x0, dg) : df{0.f, 0.f};
    p.glo[0][i] = __float2bfloat16_rn(g.lo);
    p.gf[0][i] = g.hi;
    if (dg == 0.f && col_ok) {
      const long long t = fx_of(x0.hi, wc.fx_scale) + fx_of(x0.lo, wc.fx_scale);
      if (t) atomicAdd((unsigned long long *)&bdg[c], (unsigned long long)t);
    }
  }
  __syncthreads();
  for (int c = threadIdx.x; c < kt; c += blockDim.x)
    if (bdg[c]) atomicAdd((unsigned long long *)&p.sums[c * 4 + 0], (unsigned long long)bdg[c]);
}

// Tiled forms for caller start vectors and for the results.  A warp takes 32
// consecutive original node ids u0..u0+31 and one group of 32 columns: the
// set-major vectors (original order) are read or written 32 consecutive
// floats per column, the wave's rows inv_perm[u] (relabelled) 32 columns at
// a time, and a 32x32 shared-memory tile turns one into the other, so both
// sides are coalesced.
constexpr int kTile = 32;

// batch_init for caller start vectors (wc.has_x0; x0 set-major, original order)
__global__ void __launch_bounds__(kBThreads) batch_init_x0(StepParams p, const float *__restrict__ x0,
                                                           const int32_t *__restrict__ inv_perm) {
  __shared__ float tile[kBWarps][kTile][kTile + 1];  // [column][node]
  __shared__ long long bdg[kMaxKT];
  const WaveScalars wc = p.wc->s;
  const int64_t *xcol = p.wc->xcol;
  const int kt = wc.kt, groups = kt / kTile;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int c = threadIdx.x; c < kt; c += blockDim.x) bdg[c] = 0;
  __syncthreads();
  if (blockIdx.x == 0 && wid == 0) {  // padding row: gathers of padded edges read zeros
    for (int c = lane; c < kt; c += 32) {
      const int64_t i = p.n * kt + c;
      p.glo[0][i] = p.glo[1][i] = __float2bfloat16_rn(0.f);
      p.gf[0][i] = p.gf[1][i] = 0.f;
    }
  }
  const int64_t ntiles = ceil_div<int64_t>(p.n, kTile) * groups;
  long long dang = 0;  // column gr * 32 + lane of the tiles this warp handled (one group per warp pass)
  for (int64_t tw = (int64_t)blockIdx.x * kBWarps + wid; tw < ntiles; tw += (int64_t)gridDim.x * kBWarps) {
    const int gr = (int)(tw % groups);
    const int64_t u0 = (tw / groups) * kTile;
    const int64_t u = u0 + lane;
    const bool u_ok = u < p.n;
    for (int c = 0; c < kTile; ++c) {
      const int cc = gr * kTile + c;
      tile[wid][c][lane] = (cc < wc.ncols && u_ok) ? x0[xcol[cc] * p.n + u] : 0.f;
    }
    const int32_t vl = u_ok ? inv_perm[u] : 0;
    __syncwarp();
    const int jn = (int)(p.n - u0 < (int64_t)kTile ? p.n - u0 : (int64_t)kTile);
    dang = 0;
    for (int j = 0; j < jn; ++j) {
      const int64_t v = __shfl_sync(0xffffffffu, vl, j);
      const int64_t i = v * kt + gr * kTile + lane;
      const df xv = {tile[wid][lane][j], 0.f};
      const float dg = p.deg[v];
      p.acc[i] = make_float2(xv.hi, xv.lo);
      p.tail[i] = 0.f;
      const df g = dg > 0.f ? df_div_f(xv, dg) : df{0.f, 0.f};
      p.glo[0][i] = __float2bfloat16_rn(g.lo);
      p.gf[0][i] = g.hi;
      if (dg == 0.f) dang += fx_of(xv.hi, wc.fx_scale);
    }
    if (dang) atomicAdd((unsigned long long *)&bdg[gr * kTile + lane], (unsigned long long)dang);
    __syncwarp();
  }
  __syncthreads();
  for (int c = threadIdx.x; c < kt; c += blockDim.x)
    if (bdg[c]) atomicAdd((unsigned long long *)&p.sums[c * 4 + 0], (unsigned long long)bdg[c]);
}

// float(a.x + a.y + t) without FP64 (issued at a small fraction of the FP32
// rate on this GPU): an error-free two-sum of the large terms (Knuth), then
// the small ones.
__device__ __forceinline__ float sum3_f(float ax, float ay, float t) {
  const float s = ax + t;
  const float bb = s - ax;
  const float err = (ax - (s - bb)) + (t - bb);
  return s + (err + ay);
}

// results of the wave: out[ocol[c] * n + u] = acc + tail of row inv_perm[u]
__global__ void __launch_bounds__(kBThreads) batch_finalize_t(StepParams p, float *__restrict__ out,
                                                              const int32_t *__restrict__ inv_perm) {
  __shared__ float tile[kBWarps][kTile][kTile + 1];  // [node][column]
  const WaveScalars wc = p.wc->s;
  const int64_t *ocol = p.wc->ocol;
  const int kt = wc.kt, groups = kt / kTile;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t ntiles = ceil_div<int64_t>(p.n, kTile) * groups;
  for (int64_t tw = (int64_t)blockIdx.x * kBWarps + wid; tw < ntiles; tw += (int64_t)gridDim.x * kBWarps) {
    const int gr = (int)(tw % groups);
    if (gr * kTile >= wc.ncols) continue;
    const int64_t u0 = (tw / groups) * kTile;
    const int64_t u = u0 + lane;
    const bool u_ok = u < p.n;
    const int32_t vl = u_ok ? inv_perm[u] : 0;
    const int jn = (int)(p.n - u0 < (int64_t)kTile ? p.n - u0 : (int64_t)kTile);
    for (int j = 0; j < jn; ++j) {
      const int64_t v = __shfl_sync(0xffffffffu, vl, j);
      const int64_t i = v * kt + gr * kTile + lane;
      const float2 a = p.acc[i];
      tile[wid][j][lane] = sum3_f(a.x, a.y, p.tail[i]);
    }
    __syncwarp();
    if (u_ok) {
      const int cn = min(kTile, wc.ncols - gr * kTile);
      for (int c = 0; c < cn; ++c) out[ocol[gr * kTile + c] * p.n + u] = tile[wid][lane][c];
    }
    __syncwarp();
  }
}

// chunk plan: tasks and base blocks per row with more than `chunk` in-edges
__global__ void chunk_counts(const int64_t *rp, int32_t n_big, int chunk, int64_t *nch, int64_t *nbl) {
  for (int32_t h = blockIdx.x * blockDim.x + threadIdx.x; h <= n_big; h += gridDim.x * blockDim.x) {
    const int64_t d = h < n_big ? rp[h + 1] - rp[h] : 0;
    nch[h] = ceil_div<int64_t>(d, chunk);
    nbl[h] = ceil_div<int64_t>(d, kBase);
  }
}

__global__ void chunk_fill(const int64_t *first64, const int64_t *blk64, int32_t n_big, int32_t *first,
                           int32_t *task_row, int32_t *blk) {
  for (int32_t h = blockIdx.x * blockDim.x + threadIdx.x; h <= n_big; h += gridDim.x * blockDim.x) {
    first[h] = (int32_t)first64[h];
    blk[h] = (int32_t)blk64[h];
    if (h < n_big)
      for (int64_t t = first64[h]; t < first64[h + 1]; ++t) task_row[t] = h;
  }
}

// first row with in-degree <= chunk (rows are in non-increasing degree)
__global__ void count_big(const int64_t *rp, int64_t n, int chunk, int64_t *out) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) / 2;
    if (rp[mid + 1] - rp[mid] > chunk) lo = mid + 1;
    else hi = mid;
  }
  *out = lo;
}

// prow[v] = first entry whose row >= v (entries sorted by row): a thread per
// row and a binary search (a wave has a few hundred entries over n rows, so
// a thread per entry filling its gap would leave one thread ~n writes); the
// entries are staged in shared memory when they fit (kProwStage)
constexpr int kProwStage = 4096;
__global__ void __launch_bounds__(256) prow_from_sorted(const int32_t *rows, int64_t e, int64_t n, int32_t *prow) {
  __shared__ int32_t srows[kProwStage];
  const bool staged = e <= kProwStage;
  if (staged) {
    for (int i = threadIdx.x; i < (int)e; i += blockDim.x) srows[i] = rows[i];
    __syncthreads();
  }
  const int32_t *r = staged ? srows : rows;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = e;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if ((int64_t)r[mid] < v) lo = mid + 1;
      else hi = mid;
    }
    prow[v] = (int32_t)lo;
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int cpl_index(int cpl) { return cpl == 1 ? 0 : (cpl == 2 ? 1 : 2); }

size_t block_bytes_per_col(int64_t n) {  // glo x2, gf x2, acc, tail
  return (size_t)(n + 1) * (2 * sizeof(__nv_bfloat16) + 2 * sizeof(float) + sizeof(float2) + sizeof(float));
}

Status batch_prepare_impl(Ctx *ctx, Graph *g);

// The batched state of a graph (everything but the tile workspace), built
// on first use; a failed build leaves no partial state behind.
Status batch_prepare(Ctx *ctx, Graph *g) {
  if (g->batch) return Status::ok();
  Status st = batch_prepare_impl(ctx, g);
  if (st.code != GOPS_OK) {
    cudaStreamSynchronize(ctx->stream);
    batch_free(*g);
  }
  return st;
}

// out[0] += rows with an in-edge, out[1] = min(out[1], first row without
// one); rows are below 2^31, so the warp reductions run on 32 bits
__global__ void nonempty_rows(const int64_t *rp, int64_t n, unsigned long long *out) {
  unsigned c = 0, first = ~0u;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    if (rp[v + 1] > rp[v]) ++c;
    else if ((unsigned)v < first) first = (unsigned)v;
  }
  c = __reduce_add_sync(0xffffffffu, c);
  first = __reduce_min_sync(0xffffffffu, first);
  if ((threadIdx.x & 31) == 0) {
    if (c) atomicAdd(&out[0], (unsigned long long)c);
    if (first != ~0u) atomicMin(&out[1], (unsigned long long)first);
  }
}

Status batch_prepare_impl(Ctx *ctx, Graph *g) {
  cudaStream_t s = ctx->stream;
  BatchState *b = new BatchState();
  g->batch = b;
  const int64_t n = g->n;
  b->n = n;
  GOPS_CUDA_TRY(cudaDeviceGetAttribute(&b->l2_bytes, cudaDevAttrL2CacheSize, g->device));
  GOPS_CUDA_TRY(cudaMallocHost(&b->hwave, 2 * sizeof(WaveState)));
  GOPS_CUDA_TRY(cudaEventCreateWithFlags(&b->wev[0], cudaEventDisableTiming));
  GOPS_CUDA_TRY(cudaEventCreateWithFlags(&b->wev[1], cudaEventDisableTiming));
  GOPS_CUDA_TRY(cudaMalloc(&b->sums, sizeof(long long) * 3 * kMaxKT * 4));
  GOPS_CUDA_TRY(cudaMalloc(&b->cols, sizeof(ColState) * kMaxKT));
  GOPS_CUDA_TRY(cudaMalloc(&b->wave, sizeof(WaveState)));
  GOPS_CUDA_TRY(cudaMalloc(&b->wc, sizeof(WaveConst)));
  GOPS_CUDA_TRY(cudaMalloc(&b->prow, sizeof(int32_t) * (n + 1)));
  // rows with an in-edge: a prefix of the in-degree order (if the count and
  // the first empty row disagree, nothing is skipped)
  {
    unsigned long long *d = nullptr, h[2] = {0, ~0ull};
    GOPS_CUDA_TRY(cudaMalloc(&d, sizeof(h)));
    cudaError_t e = cudaMemcpyAsync(d, h, sizeof(h), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && n > 0) {
      nonempty_rows<<<blocks_for(n, 256, ctx->num_sms * 8), 256, 0, s>>>(g->in_rp, n, d);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d);
    GOPS_CUDA_TRY(e);
    b->n_nz = (int32_t)(h[1] == h[0] ? h[0] : (unsigned long long)n);
  }
  // host copy of the relabelling, inverted
  std::vector<int32_t> perm((size_t)n);
  GOPS_CUDA_TRY(cudaMemcpyAsync(perm.data(), g->perm, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  b->inv_perm.assign((size_t)n, 0);
  for (int64_t i = 0; i < n; ++i) b->inv_perm[(size_t)perm[(size_t)i]] = (int32_t)i;
  GOPS_CUDA_TRY(cudaMalloc(&b->d_inv_perm, sizeof(int32_t) * (size_t)std::max<int64_t>(n, 1)));
  if (n > 0)
    GOPS_CUDA_TRY(cudaMemcpyAsync(b->d_inv_perm, b->inv_perm.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
  GOPS_CUDA_TRY(cudaStreamSynchronize(s));
  return Status::ok();
}

template <int CPL>
void set_grids(const Ctx *ctx, BatchState *b);

// The chunk plan for `chunk` and the blocks for k-tile 32 * cpl (kept when
// they already serve it).
Status ensure_tile(Ctx *ctx, Graph *g, int cpl, int chunk) {
  BatchState *b = g->batch;
  cudaStream_t s = ctx->stream;
  const int64_t n = g->n;
  const int kt = 32 * cpl;
  if (b->chunk != chunk) {
    free_graphs(b);
    GOPS_CUDA_TRY(cudaStreamSynchronize(s));
    free_plan(b);
    int64_t *tmp = nullptr;
    GOPS_CUDA_TRY(dev_malloc_async((void **)&tmp, sizeof(int64_t) * 2, s));
    count_big<<<1, 1, 0, s>>>(g->in_rp, n, chunk, tmp);
    int64_t nbig = 0;
    GOPS_CUDA_TRY(cudaMemcpyAsync(&nbig, tmp, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    GOPS_CUDA_TRY(cudaStreamSynchronize(s));
    free_async(tmp, s);
    int64_t tasks = 0, blocks = 0;
    GOPS_CUDA_TRY(cudaMalloc(&b->big_first, sizeof(int32_t) * (nbig + 1)));
    GOPS_CUDA_TRY(cudaMalloc(&b->blk_first, sizeof(int32_t) * (nbig + 1)));
    if (nbig > 0) {
      int64_t *nch = nullptr, *nbl = nullptr;
      GOPS_CUDA_TRY(dev_malloc_async((void **)&nch, sizeof(int64_t) * (nbig + 1), s));
      GOPS_CUDA_TRY(dev_malloc_async((void **)&nbl, sizeof(int64_t) * (nbig + 1), s));
      chunk_counts<<<blocks_for(nbig + 1, 256, 4096), 256, 0, s>>>(g->in_rp, (int32_t)nbig, chunk, nch, nbl);
      GOPS_TRY(exclusive_scan_i64(nch, nch, nbig + 1, s));
      GOPS_TRY(exclusive_scan_i64(nbl, nbl, nbig + 1, s));
      GOPS_CUDA_TRY(cudaMemcpyAsync(&tasks, nch + nbig, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
      GOPS_CUDA_TRY(cudaMemcpyAsync(&blocks, nbl + nbig, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
      GOPS_CUDA_TRY(cudaStreamSynchronize(s));
      GOPS_CUDA_TRY(cudaMalloc(&b->big_task_row, sizeof(int32_t) * std::max<int64_t>(tasks, 1)));
      chunk_fill<<<blocks_for(nbig + 1, 256, 4096), 256, 0, s>>>(nch, nbl, (int32_t)nbig, b->big_first,
                                                                  b->big_task_row, b->blk_first);
      GOPS_CUDA_TRY(cudaGetLastError());
      free_async(nch, s);
      free_async(nbl, s);
    } else {
      GOPS_CUDA_TRY(cudaMemsetAsync(b->big_first, 0, sizeof(int32_t), s));
      GOPS_CUDA_TRY(cudaMemsetAsync(b->blk_first, 0, sizeof(int32_t), s));
      GOPS_CUDA_TRY(cudaMalloc(&b->big_task_row, sizeof(int32_t)));
    }
    GOPS_CUDA_TRY(cudaMalloc(&b->lcnt, sizeof(unsigned) * (size_t)std::max<int64_t>(nbig, 1)));
    GOPS_CUDA_TRY(cudaMemsetAsync(b->lcnt, 0, sizeof(unsigned) * (size_t)std::max<int64_t>(nbig, 1), s));
    b->n_big = (int32_t)nbig;
    b->n_big_tasks = (int32_t)tasks;
    b->n_blocks = (int32_t)blocks;
    b->chunk = chunk;
    cudaFree(b->lpart);  // sized by the blocks of this plan
    b->lpart = nullptr;
  }
  if (b->kt_cap < kt) {
    free_graphs(b);
    GOPS_CUDA_TRY(cudaStreamSynchronize(s));
    free_blocks(b);
    const size_t blk = (size_t)(n + 1) * kt;
    GOPS_CUDA_TRY(cudaMalloc(&b->glo[0], sizeof(__nv_bfloat16) * blk));
    GOPS_CUDA_TRY(cudaMalloc(&b->glo[1], sizeof(__nv_bfloat16) * blk));
    GOPS_CUDA_TRY(cudaMalloc(&b->gf[0], sizeof(float) * blk));
    GOPS_CUDA_TRY(cudaMalloc(&b->gf[1], sizeof(float) * blk));
    GOPS_CUDA_TRY(cudaMalloc(&b->acc, sizeof(float2) * blk));
    GOPS_CUDA_TRY(cudaMalloc(&b->tail, sizeof(float) * blk));
    b->kt_cap = kt;
  }
  if (!b->lpart)
    GOPS_CUDA_TRY(cudaMalloc(&b->lpart, sizeof(float2) * (size_t)std::max<int32_t>(b->n_blocks, 1) * b->kt_cap));
  b->cpl = cpl;
  if (cpl == 1) set_grids<1>(ctx, b);
  else if (cpl == 2) set_grids<2>(ctx, b);
  else set_grids<4>(ctx, b);
  return Status::ok();
}

Status ensure_entries(BatchState *b, int64_t e, cudaStream_t st) {
  if (e <= b->pcap) return Status::ok();
  GOPS_CUDA_TRY(cudaStreamSynchronize(st));  // earlier waves may still read the old arrays
  free_graphs(b);                            // the captured chunks name the old arrays
  cudaFree(b->pslot); cudaFree(b->pval); cudaFree(b->prows_sorted); cudaFree(b->srow);
  b->pslot = nullptr; b->pval = nullptr; b->prows_sorted = nullptr; b->srow = nullptr;
  b->pcap = 0;  // a failed allocation below leaves no capacity claimed
  const int64_t cap = std::max<int64_t>(e, 4096);
  GOPS_CUDA_TRY(cudaMalloc(&b->pslot, sizeof(int32_t) * cap));
  GOPS_CUDA_TRY(cudaMalloc(&b->pval, sizeof(float2) * cap));
  GOPS_CUDA_TRY(cudaMalloc(&b->prows_sorted, sizeof(int32_t) * cap));
  GOPS_CUDA_TRY(cudaMalloc(&b->srow, sizeof(int32_t) * cap));
  b->pcap = cap;
  return Status::ok();
}

StepParams step_params(const Graph *g, const BatchState *b) {
  StepParams p{};
  p.n = g->n;
  p.rp = g->in_rp;
  p.col = g->in_col;
  p.deg = g->deg;
  p.perm = g->perm;
  p.n_big = b->n_big;
  p.n_big_tasks = b->n_big_tasks;
  p.chunk = b->chunk;
  // the hottest rows of both gathered blocks (read and written) fit in half of L2
  const int kt = 32 * std::max(b->cpl, 1);
  p.hot = (int32_t)std::min<double>((double)g->n, 0.5 * (double)b->l2_bytes / (2.0 * kt * sizeof(float)));
  p.big_first = b->big_first;
  p.big_task_row = b->big_task_row;
  p.blk_first = b->blk_first;
  p.prow = b->prow;
  p.pslot = b->pslot;
  p.pval = b->pval;
  p.n_nz = b->n_nz;
  p.srow = b->srow;
  p.glo[0] = b->glo[0];
  p.glo[1] = b->glo[1];
  p.gf[0] = b->gf[0];
  p.gf[1] = b->gf[1];
  p.acc = b->acc;
  p.tail = b->tail;
  p.lpart = b->lpart;
  p.lcnt = b->lcnt;
  p.sums = b->sums;
  p.cols = b->cols;
  p.wave = b->wave;
  p.wc = b->wc;
  return p;
}

template <class K>
int spmm_grid(const Ctx *ctx, const BatchState *b, K kernel) {
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kBThreads, 0);
  const int64_t need = ceil_div<int64_t>(std::max<int64_t>(b->n_big_tasks + (b->n - b->n_big), 1), kBWarps);
  return (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)ctx->num_sms * std::max(occ, 1)));
}

template <int CPL>
void set_grids(const Ctx *ctx, BatchState *b) {
  b->grid_df = spmm_grid(ctx, b, spmm_mixed<CPL>);
  b->grid_f[0] = spmm_grid(ctx, b, spmm_f32<CPL, false>);
  b->grid_f[1] = spmm_grid(ctx, b, spmm_f32<CPL, true>);
}

// One step of the wave at offset j of the chunk, in the precision phase P.
template <int CPL>
Status launch_step(const BatchState *b, StepParams p, int j, bool df, cudaStream_t st) {
  p.j = j;
  if (df) {
    spmm_mixed<CPL><<<b->grid_df, kBThreads, 0, st>>>(p);
  } else {
    if (b->l2h) spmm_f32<CPL, true><<<b->grid_f[1], kBThreads, 0, st>>>(p);
    else spmm_f32<CPL, false><<<b->grid_f[0], kBThreads, 0, st>>>(p);
  }
  GOPS_CUDA_TRY(cudaGetLastError());
  return Status::ok();
}

Status launch_step_cpl(const Ctx *, const BatchState *b, const StepParams &p, int j, bool df, cudaStream_t st) {
  switch (b->cpl) {
    case 1: return launch_step<1>(b, p, j, df, st);
    case 2: return launch_step<2>(b, p, j, df, st);
    default: return launch_step<4>(b, p, j, df, st);
  }
}

// The captured chunk: kChunkSteps steps (a double-float and an FP32 launch
// each for variant 0, FP32 only for variant 1), then the step counter.
Status ensure_chunk_graph(Ctx *ctx, Graph *g, int variant) {
  BatchState *b = g->batch;
  if (b->exec_cpl != b->cpl || b->exec_chunk != b->chunk || b->exec_pslot != b->pslot || b->exec_l2h != (int)b->l2h)
    free_graphs(b);
  if (b->chunk_exec[variant]) return Status::ok();
  cudaStream_t st = ctx->stream;
  const StepParams p = step_params(g, b);
  cudaGraph_t graph = nullptr;
  GOPS_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  Status cs;
  for (int j = 0; j < kChunkSteps && cs.code == GOPS_OK; ++j) {
    if (variant == 0) cs = launch_step_cpl(ctx, b, p, j, true, st);
    if (cs.code == GOPS_OK) cs = launch_step_cpl(ctx, b, p, j, false, st);
  }
  if (cs.code == GOPS_OK) {
    advance_kernel<<<1, 1, 0, st>>>(b->wave);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) cs = Status{GOPS_ERR_CUDA, cudaGetErrorString(e)};
  }
  const cudaError_t ee = cudaStreamEndCapture(st, &graph);
  GOPS_TRY(cs);
  GOPS_CUDA_TRY(ee);
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  GOPS_CUDA_TRY(ei);
  b->chunk_exec[variant] = exec;
  b->exec_cpl = b->cpl;
  b->exec_chunk = b->chunk;
  b->exec_l2h = (int)b->l2h;
  b->exec_pslot = b->pslot;
  return Status::ok();
}

void fill_wave_const(WaveScalars &w, const gops_config *cfg, int64_t n, int kt, int ncols, bool has_x0, double wmax) {
  w.d = df_from_double(cfg->damping);
  w.omd = df_from_double(1.0 - cfg->damping);
  w.inv_n = df_from_double(1.0 / (double)n);
  w.tol = cfg->tolerance;
  w.max_iter = cfg->max_iterations;
  w.ncols = ncols;
  w.has_x0 = has_x0 ? 1 : 0;
  w.kt = kt;
  w.skip_from = INT32_MAX;  // set per wave by its caller
  w.n_srow = 0;
  // fixed-point range: a start of L1 norm up to wmax keeps every partial
  // sum far below 2^63; larger or non-finite starts are flagged by the
  // nonfinite counter and the column does not converge
  int e = 0;
  while (e < 20 && std::ldexp(1.0, e) < wmax) ++e;
  const int F = 58 - 2 * e;
  w.fx_scale = std::ldexp(1.0f, F);
  w.fx_inv = std::ldexp(1.0, -F);
}

// ---------------------------------------------------------------------------
// autotuner: the k-tile (columns per lane) and the chunk size of long rows,
// picked per graph from timed steps on a probe wave (uniform personalization
// in every column, never converging) with the workspace the choice needs;
// then, for the chosen tile, the FP32 step with and without L2 eviction
// hints.  Cost of a candidate: its time per column-step, 3/4 FP32 and 1/4
// double-float steps.  Results do not depend on the choice (canonical row
// sums, per-column precision phases; cache hints change no value), only the
// time does.
// ---------------------------------------------------------------------------
Status probe_tile(Ctx *ctx, Graph *g, int cpl, int chunk, float *cost) {
  BatchState *b = g->batch;
  cudaStream_t st = ctx->stream;
  GOPS_TRY(ensure_tile(ctx, g, cpl, chunk));
  const int kt = 32 * cpl;
  gops_config cfg{0.85, 1000000, 0.0};
  WaveConst w{};
  fill_wave_const(w.s, &cfg, g->n, kt, kt, false, 1.0);
  std::vector<ColState> cols(kMaxKT, ColState{0, 0.0, 1, 0, 1, 0, (double)INFINITY, (double)INFINITY});
  for (int c = 0; c < kt; ++c) cols[c].retired = 0;
  GOPS_CUDA_TRY(cudaMemcpyAsync(b->wc, &w, sizeof(WaveConst), cudaMemcpyHostToDevice, st));
  GOPS_CUDA_TRY(cudaMemcpyAsync(b->cols, cols.data(), sizeof(ColState) * kMaxKT, cudaMemcpyHostToDevice, st));
  GOPS_CUDA_TRY(cudaMemsetAsync(b->wave, 0, sizeof(WaveState), st));
  GOPS_CUDA_TRY(cudaMemsetAsync(b->sums, 0, sizeof(long long) * 3 * kMaxKT * 4, st));
  GOPS_CUDA_TRY(cudaMemsetAsync(b->prow, 0, sizeof(int32_t) * (g->n + 1), st));
  GOPS_CUDA_TRY(cudaMemsetAsync(b->lcnt, 0, sizeof(unsigned) * (size_t)std::max<int32_t>(b->n_big, 1), st));
  StepParams p = step_params(g, b);
  batch_init<<<blocks_for((g->n + 1) * kt, kBThreads, ctx->num_sms * 8), kBThreads, 0, st>>>(p);
  GOPS_CUDA_TRY(cudaGetLastError());
  // step 1 (double-float), then FP32 steps (theta = inf: FP32 from step 2)
  constexpr int kF = 3;
  cudaEvent_t ev[2 * (kF + 1)];
  for (auto &e : ev) GOPS_CUDA_TRY(cudaEventCreate(&e));
  struct EvGuard {
    cudaEvent_t *e; int n;
    ~EvGuard() { for (int i = 0; i < n; ++i) cudaEventDestroy(e[i]); }
  } guard{ev, 2 * (kF + 1)};
  GOPS_CUDA_TRY(cudaEventRecord(ev[0], st));
  GOPS_TRY(launch_step_cpl(ctx, b, p, 0, true, st));
  GOPS_CUDA_TRY(cudaEventRecord(ev[1], st));
  for (int i = 0; i < kF; ++i) {
    GOPS_CUDA_TRY(cudaEventRecord(ev[2 + 2 * i], st));
    GOPS_TRY(launch_step_cpl(ctx, b, p, 1 + i, false, st));
    GOPS_CUDA_TRY(cudaEventRecord(ev[3 + 2 * i], st));
  }
  GOPS_CUDA_TRY(cudaStreamSynchronize(st));
  float t_df = 0.f;
  cudaEventElapsedTime(&t_df, ev[0], ev[1]);
  std::vector<float> tf(kF);
  for (int i = 0; i < kF; ++i) cudaEventElapsedTime(&tf[i], ev[2 + 2 * i], ev[3 + 2 * i]);
  std::sort(tf.begin(), tf.end());
  *cost = (0.75f * tf[kF / 2] + 0.25f * t_df) / (float)kt;
  return Status::ok();
}

Status batch_tune(Ctx *ctx, Graph *g) {
  BatchState *b = g->batch;
  if (b->tuned) return Status::ok();
  const int chunks[2] = {256, 1024};
  int cpls[3] = {1, 2, 4};
  // the wave workspace may take ~40 % of the device memory free now
  size_t free_b = 0, total_b = 0;
  GOPS_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
  const size_t budget = (size_t)(0.4 * (double)free_b);
  float best = INFINITY;
  int best_cpl = 1, best_chunk = 256;
  for (int cpl : cpls) {
    if (cpl > 1 && block_bytes_per_col(g->n) * 32 * cpl > budget) continue;
    for (int ch : chunks) {
      float c = 0.f;
      GOPS_TRY(probe_tile(ctx, g, cpl, ch, &c));
      b->tune_ms[cpl_index(cpl)][ch == 256 ? 0 : 1] = c;
      if (c < best) {
        best = c;
        best_cpl = cpl;
        best_chunk = ch;
      }
    }
  }
  // keep only the workspace the choice needs
  if (b->kt_cap > 32 * best_cpl) {
    free_graphs(b);
    GOPS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    free_blocks(b);
  }
  b->chunk = 0;  // rebuild the plan for the chosen chunk
  free_plan(b);
  GOPS_TRY(ensure_tile(ctx, g, best_cpl, best_chunk));
  // the chosen tile's FP32 step with L2 eviction hints
  b->l2h = true;
  float c2 = 0.f;
  GOPS_TRY(probe_tile(ctx, g, best_cpl, best_chunk, &c2));
  b->tune_l2 = c2;
  b->l2h = c2 < best;
  b->tuned = true;
  return Status::ok();
}

}  // namespace

// Choose (cols > 0) or autotune (cols == 0) the k-tile, chunk size and L2 hints.
Status batch_set_tile(Ctx *ctx, Graph *g, int cols, int chunk, int l2_hints) {
  GOPS_TRY(batch_prepare(ctx, g));
  BatchState *b = g->batch;
  if (cols == 0) {
    b->tuned = false;
    return batch_tune(ctx, g);
  }
  if (cols != 32 && cols != 64 && cols != 128) return Status{GOPS_ERR_INVALID, "cols must be 0, 32, 64 or 128"};
  if (chunk < kBase || chunk % kBase) return Status{GOPS_ERR_INVALID, "chunk must be a positive multiple of 256"};
  if (b->kt_cap > cols) {
    free_graphs(b);
    GOPS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    free_blocks(b);
  }
  GOPS_TRY(ensure_tile(ctx, g, cols / 32, chunk));
  b->l2h = l2_hints != 0;
  b->tuned = true;
  return Status::ok();
}

Status batch_get_tile(Graph *g, int *cols, int *chunk, int *l2_hints, float *cost) {
  BatchState *b = g->batch;
  if (!b || !b->tuned) {
    *cols = 0;
    *chunk = 0;
    *l2_hints = 0;
    if (cost)
      for (int i = 0; i < 7; ++i) cost[i] = 0.f;
    return Status::ok();
  }
  *cols = 32 * b->cpl;
  *chunk = b->chunk;
  *l2_hints = b->l2h ? 1 : 0;
  if (cost) {
    for (int i = 0; i < 6; ++i) cost[i] = b->tune_ms[i / 2][i % 2];
    cost[6] = b->tune_l2;
  }
  return Status::ok();
}

// nsets seed sets -> scores (host or device, set-major, original node order)
Status ppr_batch(Ctx *ctx, Graph *g, const gops_config *cfg, int64_t nsets, const int64_t *seed_ptr,
                 const int32_t *seed_idx, const float *x0, bool x0_on_device, float *scores,
                 bool scores_on_device, gops_run *runs, const double *r1_max, int32_t *rejected) {
  ctx->stats = gops_stats{};
  const int64_t n = g->n;
  if (nsets <= 0) return Status::ok();
  if (n == 0) {  // src/ppr.rs:96-103
    if (runs)
      for (int64_t s = 0; s < nsets; ++s) runs[s] = gops_run{0, 0.0, 1, 0};
    return Status::ok();
  }
  for (int64_t s = 0; s < nsets; ++s)
    if (seed_ptr[s + 1] < seed_ptr[s]) return Status{GOPS_ERR_INVALID, "seed_ptr must be non-decreasing"};
  for (int64_t k = seed_ptr[0]; k < seed_ptr[nsets]; ++k)
    if (seed_idx[k] < 0 || seed_idx[k] >= n) return Status{GOPS_ERR_INVALID, "seed index out of range"};
  GOPS_TRY(batch_prepare(ctx, g));
  GOPS_TRY(batch_tune(ctx, g));
  BatchState *b = g->batch;
  cudaStream_t st = ctx->stream;
  const int KT = 32 * b->cpl;
  if (x0 && !x0_on_device && b->x0_cols < KT) {
    cudaFree(b->x0);
    b->x0 = nullptr;
    b->x0_cols = 0;
    GOPS_CUDA_TRY(cudaMalloc(&b->x0, sizeof(float) * (size_t)n * KT));
    b->x0_cols = KT;
  }
  if (scores && !scores_on_device && b->out_cols < KT) {
    cudaFree(b->out);
    b->out = nullptr;
    b->out_cols = 0;
    GOPS_CUDA_TRY(cudaMalloc(&b->out, sizeof(float) * (size_t)n * KT));
    b->out_cols = KT;
  }

  uint64_t launches = 0, col_iters = 0;
  float spmm_ms = 0.f, df_ms = 0.f;
  uint64_t spmm_launches = 0, df_launches = 0;
  // host results: each wave's block goes to a pinned buffer in one copy, and
  // host threads scatter its columns to the sets' rows while the GPU runs
  // the next wave (two buffers; a buffer's scatter is joined before reuse)
  const size_t block_bytes = sizeof(float) * (size_t)KT * (size_t)n;
  // a page-locked host destination takes every set's row by DMA straight
  // from the wave's block, on the copy stream (no staging, no host copy)
  bool direct = false;
  if (scores && !scores_on_device) {
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, scores) == cudaSuccess) direct = pa.type == cudaMemoryTypeHost;
    else cudaGetLastError();  // not a pointer CUDA knows: pageable
  }
  // copies still in flight into the caller's array end before any return
  struct CopyGuard {
    cudaStream_t s;
    bool on;
    ~CopyGuard() {
      if (on) cudaStreamSynchronize(s);
    }
  } copy_guard{ctx->copy_stream, direct};
  const bool staged = scores && !scores_on_device && !direct && block_bytes <= (size_t(1) << 31);
  // the context's pinned staging, grown when a wave's block does not fit
  if (staged && ctx->hstage_bytes < block_bytes) {
    for (auto &h : ctx->hstage)
      if (h) {
        cudaFreeHost(h);
        h = nullptr;
      }
    ctx->hstage_bytes = 0;
    GOPS_CUDA_TRY(cudaMallocHost(&ctx->hstage[0], block_bytes));
    GOPS_CUDA_TRY(cudaMallocHost(&ctx->hstage[1], block_bytes));
    ctx->hstage_bytes = block_bytes;
  }
  if ((staged || direct) && !ctx->sev[0]) {
    GOPS_CUDA_TRY(cudaEventCreateWithFlags(&ctx->sev[0], cudaEventDisableTiming));
    GOPS_CUDA_TRY(cudaEventCreateWithFlags(&ctx->sev[1], cudaEventDisableTiming));
  }
  constexpr int kScatterThreads = 4;
  struct Scatter {
    std::vector<std::thread> t[2];
    void join(int q) {
      for (auto &x : t[q])
        if (x.joinable()) x.join();
      t[q].clear();
    }
    ~Scatter() { join(0); join(1); }
  } scatter;

  // waves of sets of similar size: a set's step count falls with its size,
  // and a wave runs until its slowest column retires
  std::vector<int64_t> order(nsets);
  for (int64_t q = 0; q < nsets; ++q) order[q] = q;
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t c) {
    return seed_ptr[a + 1] - seed_ptr[a] < seed_ptr[c + 1] - seed_ptr[c];
  });
  // a wave whose block is being copied to hstage[q] and not yet scattered:
  // its scatter starts once the copy's event has passed, while the next wave
  // runs on the device (no stream synchronisation at the wave boundary)
  struct PendingScatter {
    int64_t set0 = -1;
    int ncols = 0, q = 0;
  } pend;
  int pend_copy_q = -1;  // the last wave whose block went to a pinned buffer
  auto start_scatter = [&]() -> Status {
    if (pend.set0 < 0) return Status::ok();
    GOPS_CUDA_TRY(cudaEventSynchronize(ctx->sev[pend.q]));
    const float *src = ctx->hstage[pend.q];
    const int ncols_p = pend.ncols;
    const std::vector<int64_t> ids(order.begin() + pend.set0, order.begin() + pend.set0 + ncols_p);
    for (int t = 0; t < kScatterThreads; ++t)
      scatter.t[pend.q].emplace_back([=]() {
        for (int c = t; c < ncols_p; c += kScatterThreads)
          std::memcpy(scores + ids[c] * n, src + (size_t)c * n, sizeof(float) * (size_t)n);
      });
    pend.set0 = -1;
    return Status::ok();
  };
  // Host side of a wave (personalization entries, column records), built for
  // wave w+1 while wave w runs on the device.
  struct HostWave {
    int ncols = 0;
    bool uniform = false;  // some column has the uniform personalization
    std::vector<ColState> cols;
    std::vector<int32_t> erow, eslot, srow;
    std::vector<float2> eval;
  } hw[2];
  auto prep = [&](HostWave &h, int64_t set0) {
    h.ncols = (int)std::min<int64_t>(KT, nsets - set0);
    h.cols.assign(kMaxKT, ColState{});
    std::map<std::pair<int32_t, int32_t>, double> ent;
    for (int c = 0; c < kMaxKT; ++c) {
      const double r1 = r1_max && c < h.ncols ? r1_max[order[set0 + c]] : (double)INFINITY;
      h.cols[c] = ColState{0, 0.0, c < h.ncols ? 0 : 1, 0, 0, 0, r1,
                           x0 && std::isfinite(r1) ? kBThetaWarm : kBTheta};
    }
    h.uniform = false;
    for (int c = 0; c < h.ncols; ++c) {
      const int64_t a0 = seed_ptr[order[set0 + c]], a1 = seed_ptr[order[set0 + c] + 1];
      if (a1 == a0) {  // sum <= 0: uniform (src/ppr.rs:108)
        h.cols[c].uniform = 1;
        h.uniform = true;
        continue;
      }
      const double inv = 1.0 / (double)(a1 - a0);
      for (int64_t k = a0; k < a1; ++k) ent[{b->inv_perm[(size_t)seed_idx[k]], c}] += inv;
    }
    h.erow.clear(); h.eslot.clear(); h.eval.clear(); h.srow.clear();
    for (const auto &kv : ent) {  // by row, then column
      const int32_t r = kv.first.first;
      h.erow.push_back(r);
      h.eslot.push_back(kv.first.second);
      const df w = df_from_double(kv.second);
      h.eval.push_back(make_float2(w.hi, w.lo));
      if (r >= b->n_nz && (h.srow.empty() || h.srow.back() != r)) h.srow.push_back(r);
    }
  };
  // per-column records of every wave stay on the device until the end
  const int64_t nwaves = ceil_div<int64_t>(nsets, KT);
  ColState *cols_all = nullptr;
  GOPS_CUDA_TRY(dev_malloc_async((void **)&cols_all, sizeof(ColState) * (size_t)nwaves * KT, st));
  struct FreeOnExit {
    void *p; cudaStream_t s;
    ~FreeOnExit() { free_async(p, s); }
  } cols_all_guard{cols_all, st};
  // the largest entry count of any wave, so that the entry arrays (named by
  // the captured chunks) are sized once per call
  {
    int64_t emax = 0;
    for (int64_t set0 = 0; set0 < nsets; set0 += KT) {
      int64_t e = 0;
      for (int64_t q = set0; q < std::min<int64_t>(nsets, set0 + KT); ++q) e += seed_ptr[order[q] + 1] - seed_ptr[order[q]];
      emax = std::max(emax, e);
    }
    GOPS_TRY(ensure_entries(b, emax, st));
  }
  const bool use_graphs = !ctx->timing;
  if (use_graphs) {
    GOPS_TRY(ensure_chunk_graph(ctx, g, 0));
    GOPS_TRY(ensure_chunk_graph(ctx, g, 1));
  }
  StepParams p = step_params(g, b);
  prep(hw[0], 0);
  GOPS_CUDA_TRY(cudaEventRecord(ctx->ev[0], st));
  for (int64_t set0 = 0; set0 < nsets; set0 += KT) {
    HostWave &h = hw[(set0 / KT) & 1];
    const int ncols = h.ncols;
    // ---- per-wave constants (a small pageable copy: staged at the call)
    WaveConst w{};
    fill_wave_const(w.s, cfg, n, KT, ncols, x0 != nullptr, x0 ? 8.0 : 1.0);
    for (int c = 0; c < kMaxKT; ++c) {
      const int64_t sid = c < ncols ? order[set0 + c] : 0;
      w.xcol[c] = x0 && !x0_on_device ? c : sid;
      w.ocol[c] = scores && !scores_on_device ? c : sid;
    }
    w.s.skip_from = h.uniform ? INT32_MAX : x0 ? kSkipFromWarm : kSkipFromCold;
    w.s.n_srow = (int)h.srow.size();
    if (!h.srow.empty())
      GOPS_CUDA_TRY(cudaMemcpyAsync(b->srow, h.srow.data(), sizeof(int32_t) * h.srow.size(), cudaMemcpyHostToDevice,
                                    st));
    const int64_t ne = (int64_t)h.erow.size();
    if (ne) {
      GOPS_CUDA_TRY(cudaMemcpyAsync(b->prows_sorted, h.erow.data(), sizeof(int32_t) * ne, cudaMemcpyHostToDevice, st));
      GOPS_CUDA_TRY(cudaMemcpyAsync(b->pslot, h.eslot.data(), sizeof(int32_t) * ne, cudaMemcpyHostToDevice, st));
      GOPS_CUDA_TRY(cudaMemcpyAsync(b->pval, h.eval.data(), sizeof(float2) * ne, cudaMemcpyHostToDevice, st));
      ctx->stats.h2d_bytes += (sizeof(int32_t) * 2 + sizeof(float2)) * ne;
    }
    prow_from_sorted<<<blocks_for(n + 1, 256, ctx->num_sms * 8), 256, 0, st>>>(b->prows_sorted, ne, n, b->prow);
    ++launches;
    // ---- warm start of the wave
    const float *x0w = nullptr;
    if (x0) {
      if (x0_on_device) {
        x0w = x0;
      } else {
        for (int c = 0; c < ncols; ++c)
          GOPS_CUDA_TRY(cudaMemcpyAsync(b->x0 + (size_t)c * n, x0 + order[set0 + c] * n, sizeof(float) * (size_t)n,
                                        cudaMemcpyHostToDevice, st));
        ctx->stats.h2d_bytes += sizeof(float) * (size_t)ncols * n;
        x0w = b->x0;
      }
    }
    GOPS_CUDA_TRY(cudaMemcpyAsync(b->wc, &w, sizeof(WaveConst), cudaMemcpyHostToDevice, st));
    GOPS_CUDA_TRY(cudaMemcpyAsync(b->cols, h.cols.data(), sizeof(ColState) * kMaxKT, cudaMemcpyHostToDevice, st));
    GOPS_CUDA_TRY(cudaMemsetAsync(b->wave, 0, sizeof(WaveState), st));
    GOPS_CUDA_TRY(cudaMemsetAsync(b->sums, 0, sizeof(long long) * 3 * kMaxKT * 4, st));
    if (x0w)
      batch_init_x0<<<blocks_for(ceil_div<int64_t>(n, kTile) * (KT / kTile), kBWarps, ctx->num_sms * 8), kBThreads, 0,
                      st>>>(p, x0w, b->d_inv_perm);
    else
      batch_init<<<blocks_for((n + 1) * KT, kBThreads, ctx->num_sms * 8), kBThreads, 0, st>>>(p);
    GOPS_CUDA_TRY(cudaGetLastError());
    ++launches;
    // ---- steps: chunks of kChunkSteps launches; one chunk stays queued
    // ahead of the host's poll of the wave record, so the GPU does not wait
    // for the host between chunks (a step launched after the wave is done
    // returns in its prologue)
    bool f32_known = false;
    unsigned long long k = 1;  // next step to launch
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> evs;
    std::vector<std::pair<unsigned long long, bool>> evk;
    auto launch_chunk = [&]() -> Status {
      if (use_graphs) {
        GOPS_CUDA_TRY(cudaGraphLaunch(b->chunk_exec[f32_known ? 1 : 0], st));
        launches += (f32_known ? 1 : 2) * kChunkSteps + 1;
      } else {
        for (int j = 0; j < kChunkSteps; ++j) {
          for (int v = f32_known ? 1 : 0; v < 2; ++v) {
            const bool isdf = v == 0;
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            GOPS_CUDA_TRY(cudaEventCreate(&e0));
            GOPS_CUDA_TRY(cudaEventCreate(&e1));
            GOPS_CUDA_TRY(cudaEventRecord(e0, st));
            GOPS_TRY(launch_step_cpl(ctx, b, p, j, isdf, st));
            GOPS_CUDA_TRY(cudaEventRecord(e1, st));
            evs.push_back({e0, e1});
            evk.push_back({k + j, isdf});
            ++launches;
          }
        }
        advance_kernel<<<1, 1, 0, st>>>(b->wave);
        GOPS_CUDA_TRY(cudaGetLastError());
        ++launches;
      }
      k += kChunkSteps;
      return Status::ok();
    };
    auto poll_after = [&](int slot) -> Status {
      GOPS_CUDA_TRY(cudaMemcpyAsync(&b->hwave[slot], b->wave, sizeof(WaveState), cudaMemcpyDeviceToHost, st));
      GOPS_CUDA_TRY(cudaEventRecord(b->wev[slot], st));
      return Status::ok();
    };
    int pending[2], npend = 0;
    for (int q = 0; q < 2 && k - 1 <= cfg->max_iterations; ++q) {
      GOPS_TRY(launch_chunk());
      GOPS_TRY(poll_after(q));
      pending[npend++] = q;
    }
    GOPS_TRY(start_scatter());  // the previous wave's block, while this wave runs
    if (set0 + KT < nsets) prep(hw[((set0 / KT) + 1) & 1], set0 + KT);  // overlaps this wave
    bool finished = false;
    while (npend > 0) {
      const int slot = pending[0];
      pending[0] = pending[1];
      --npend;
      GOPS_CUDA_TRY(cudaEventSynchronize(b->wev[slot]));
      const WaveState ws = b->hwave[slot];
      if (ws.done) {
        GOPS_CUDA_TRY(cudaStreamSynchronize(st));
        // time the launches that did work (their step <= steps, in their phase)
        for (size_t i = 0; i < evs.size(); ++i) {
          const unsigned long long kk = evk[i].first;
          const bool isdf = evk[i].second;
          const bool did = kk <= ws.steps &&
                           (isdf ? (ws.f32_from == 0 || kk < ws.f32_from) : (ws.f32_from && kk >= ws.f32_from));
          if (did) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, evs[i].first, evs[i].second);
            if (isdf) { df_ms += ms; ++df_launches; }
            else { spmm_ms += ms; ++spmm_launches; }
          }
        }
        for (auto &pr : evs) { cudaEventDestroy(pr.first); cudaEventDestroy(pr.second); }
        finished = true;
        break;
      }
      if (ws.f32_phase) f32_known = true;
      if (k - 1 <= cfg->max_iterations) {
        GOPS_TRY(launch_chunk());
        GOPS_TRY(poll_after(slot));
        pending[npend++] = slot;
      }
    }
    if (!finished) return Status{GOPS_ERR_INTERNAL, "wave did not finish"};
    // ---- results of the wave
    if (scores) {
      float *outw = scores_on_device ? scores : b->out;
      // the previous wave's copies (on the copy stream) have read b->out
      if ((staged || direct) && pend_copy_q >= 0) GOPS_CUDA_TRY(cudaStreamWaitEvent(st, ctx->sev[pend_copy_q], 0));
      batch_finalize_t<<<blocks_for(ceil_div<int64_t>(n, kTile) * (KT / kTile), kBWarps, ctx->num_sms * 8), kBThreads,
                         0, st>>>(p, outw, b->d_inv_perm);
      GOPS_CUDA_TRY(cudaGetLastError());
      ++launches;
      if (direct) {
        // one copy per set into the caller's page-locked array, on the copy
        // stream, overlapping the next wave's steps
        GOPS_CUDA_TRY(cudaEventRecord(ctx->copy_ev[0], st));
        GOPS_CUDA_TRY(cudaStreamWaitEvent(ctx->copy_stream, ctx->copy_ev[0], 0));
        for (int c = 0; c < ncols; ++c)
          GOPS_CUDA_TRY(cudaMemcpyAsync(scores + order[set0 + c] * n, b->out + (size_t)c * n, sizeof(float) * (size_t)n,
                                        cudaMemcpyDeviceToHost, ctx->copy_stream));
        GOPS_CUDA_TRY(cudaEventRecord(ctx->sev[0], ctx->copy_stream));
        pend_copy_q = 0;
        ctx->stats.d2h_bytes += sizeof(float) * (size_t)ncols * n;
      } else if (staged) {
        // the copy to the pinned buffer runs on the copy stream, overlapping
        // the next wave's steps
        const int q = (int)((set0 / KT) & 1);
        scatter.join(q);  // the scatter of two waves ago read this buffer
        GOPS_CUDA_TRY(cudaEventRecord(ctx->copy_ev[0], st));
        GOPS_CUDA_TRY(cudaStreamWaitEvent(ctx->copy_stream, ctx->copy_ev[0], 0));
        GOPS_CUDA_TRY(cudaMemcpyAsync(ctx->hstage[q], b->out, sizeof(float) * (size_t)ncols * n,
                                      cudaMemcpyDeviceToHost, ctx->copy_stream));
        GOPS_CUDA_TRY(cudaEventRecord(ctx->sev[q], ctx->copy_stream));
        pend_copy_q = q;
        ctx->stats.d2h_bytes += sizeof(float) * (size_t)ncols * n;
        pend.set0 = set0;
        pend.ncols = ncols;
        pend.q = q;
      } else if (!scores_on_device) {
        for (int c = 0; c < ncols; ++c)
          GOPS_CUDA_TRY(cudaMemcpyAsync(scores + order[set0 + c] * n, b->out + (size_t)c * n, sizeof(float) * (size_t)n,
                                        cudaMemcpyDeviceToHost, st));
        ctx->stats.d2h_bytes += sizeof(float) * (size_t)ncols * n;
      }
    }
    GOPS_CUDA_TRY(cudaMemcpyAsync(cols_all + (set0 / KT) * KT, b->cols, sizeof(ColState) * KT,
                                  cudaMemcpyDeviceToDevice, st));
  }
  GOPS_TRY(start_scatter());  // the last wave's block
  if (direct && pend_copy_q >= 0) GOPS_CUDA_TRY(cudaStreamWaitEvent(st, ctx->sev[0], 0));
  std::vector<ColState> cols_res((size_t)nwaves * KT);
  GOPS_CUDA_TRY(cudaMemcpyAsync(cols_res.data(), cols_all, sizeof(ColState) * cols_res.size(), cudaMemcpyDeviceToHost,
                                st));
  GOPS_CUDA_TRY(cudaStreamSynchronize(st));
  for (int64_t set0 = 0; set0 < nsets; set0 += KT) {
    const int ncols = (int)std::min<int64_t>(KT, nsets - set0);
    const ColState *cr = cols_res.data() + (set0 / KT) * KT;
    for (int c = 0; c < ncols; ++c) {
      col_iters += cr[c].iterations;
      if (runs) runs[order[set0 + c]] = gops_run{cr[c].iterations, cr[c].diff_l1, cr[c].converged, 0};
      if (rejected) rejected[order[set0 + c]] = cr[c].rejected;
    }
  }
  scatter.join(0);
  scatter.join(1);
  GOPS_CUDA_TRY(cudaEventRecord(ctx->ev[3], st));
  GOPS_CUDA_TRY(cudaEventSynchronize(ctx->ev[3]));
  float t_all = 0.f;
  cudaEventElapsedTime(&t_all, ctx->ev[0], ctx->ev[3]);
  ctx->stats.solve_ms = t_all;
  ctx->stats.kernel_launches = launches;
  ctx->stats.iterations = col_iters;
  ctx->stats.f32_ms = spmm_ms;
  ctx->stats.f32_launches = spmm_launches;
  ctx->stats.df_ms = df_ms;
  ctx->stats.df_launches = df_launches;
  return Status::ok();
}

}  // namespace gops
