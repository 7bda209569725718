// Graph ingestion on the device.
//
//  K1  out-adjacency (adapter order) -> in-edge CSR: a stable radix sort of
//      edge ids by destination (read from the uploaded columns), so every
//      in-row lists its sources in ascending source order, the order the
//      reference scatters in (src/pagerank.rs:154-162); in-row offsets come
//      from the sorted keys (no atomics on hub destinations).  Per out-row:
//      source ids and out-degree (structure pass, before the weights have
//      arrived), then weight sum sum max(w,0) and transition weights
//      max(w,0)/sum (replacing the neighbor / out_wsum precompute of
//      src/pagerank.rs:136-137,226-234 and src/ppr.rs:112).
//  K2  relabelling and the pull kernels' plan: a stable radix sort of nodes by
//      in-degree (descending) gives perm; the in-edge CSR is rewritten in that
//      order with relabelled sources; rows then fall into contiguous degree
//      classes (segments), each processed with one sub-warp width, and rows
//      above kHubThreshold in-edges are split into kHubChunk-edge warp tasks.
//  Dense  AdjacencyMatrix (src/graph.rs:128-141) -> out-CSR by a warp-ballot
//      compaction of each matrix row (entries > 0.0, ascending column).
#include <algorithm>

#include "objects.cuh"
#include "primitives.cuh"

namespace gops {

namespace {

// Per out-row u: out-degree and the source id of every entry (the structure
// pass, before the weights have arrived), then (weighted) the transition
// weight max(w,0) / sum_u max(w,0) in FP32 with the weighted-dangling bit.
// FP64 instructions issue at a small fraction of the FP32 rate on this GPU,
// so the weight passes keep them to one add per entry, one divide per row and
// one multiply and conversion per entry:
//  out_rows          structure pass, rows of at most kRowBig entries (nearly
//                    all: R-MAT rows average ~16): an 8-lane group per row;
//                    longer rows are listed in
//                    big[1..big[0]] (list order varies, results do not)
//  out_rows_big      structure pass, the listed rows (hubs), a block per row
//  row_sums_tiles    the sums over the entry array in 256-entry warp tiles
//                    (every lane sums 8 consecutive entries in order), pieces
//                    of a row joined across lanes and tiles in a fixed order
//  row_finish        a thread per row: the row's pieces -> sum -> 1/sum (0 for
//                    an empty or zero-weight row) and the dangling bits
//  edge_weights      a thread per entry: (float)(max(w,0) * inverse of its row),
//                    stored beside the entry's source so that the in-CSR
//                    scatter gathers both with one 8-byte load
constexpr int kRowLanes = 8;
constexpr int64_t kRowBig = 256;

// max(w, 0), 0 for NaN (the maximum ignores a NaN operand), from the bits
__device__ __forceinline__ double clamp_weight(double w) {
  const long long b = __double_as_longlong(w);
  const bool neg_or_nan = b < 0 || b > 0x7ff0000000000000LL;  // sign set, or NaN
  return neg_or_nan ? 0.0 : w;
}

__global__ void out_rows(int64_t n, const int64_t *__restrict__ rp, uint32_t *__restrict__ src,
                         float *__restrict__ deg_f, uint32_t *__restrict__ big) {
  const int lane = threadIdx.x & (kRowLanes - 1);
  const int64_t groups = (int64_t)gridDim.x * (blockDim.x / kRowLanes);
  for (int64_t u = (int64_t)blockIdx.x * (blockDim.x / kRowLanes) + threadIdx.x / kRowLanes; u < n; u += groups) {
    const int64_t b = rp[u], e = rp[u + 1];
    if (e - b > kRowBig) {  // the whole group skips: same row
      if (lane == 0) big[1 + atomicAdd(&big[0], 1u)] = (uint32_t)u;
      continue;
    }
    if (lane == 0) deg_f[u] = (float)(e - b);
    for (int64_t i = b + lane; i < e; i += kRowLanes) src[i] = (uint32_t)u;
  }
}

__global__ void __launch_bounds__(256) out_rows_big(const int64_t *__restrict__ rp, uint32_t *__restrict__ src,
                                                     float *__restrict__ deg_f, const uint32_t *__restrict__ big) {
  const uint32_t nbig = big[0];
  for (uint32_t k = blockIdx.x; k < nbig; k += gridDim.x) {
    const int64_t u = big[1 + k];
    const int64_t b = rp[u], e = rp[u + 1];
    if (threadIdx.x == 0) deg_f[u] = (float)(e - b);
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) src[i] = (uint32_t)u;
  }
}

// The sums pass.  Warp tile t holds entries [256 t, 256 t + 256), lane l the
// 8 from 256 t + 8 l.  A lane adds its entries in order, row by row (src
// gives each entry's row); a row begun and ended in the lane is written to
// rowsum.  A row that crosses lanes is joined by a segmented scan over the
// lanes (left to right): the lane where it ends adds the scan's carry from
// the left to its own first piece.  A row that crosses the tile's ends
// leaves its pieces for row_finish: tcarry[t] = the part in tile t of the
// tile's last row, when that row continues past the tile (a tile inside one
// row: the tile's sum), thead[t] = the part in tile t of the tile's first
// row, when that row began before the tile and ends in it.  One FP64 add per
// entry and a few per tile; the order is fixed by the tiling.
constexpr int kSumItems = 8;
constexpr int kSumTile = 32 * kSumItems;
constexpr uint32_t kNoRow = 0xFFFFFFFFu;

__global__ void __launch_bounds__(256) row_sums_tiles(int64_t m, const uint32_t *__restrict__ src,
                                                       const double *__restrict__ w, int vec,
                                                       double *__restrict__ rowsum, double *__restrict__ tcarry,
                                                       double *__restrict__ thead) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int64_t t = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int64_t T = t * kSumTile;
  if (T >= m) return;  // the whole warp
  const int64_t i0 = T + (int64_t)lane * kSumItems;
  uint32_t r[kSumItems];
  double x[kSumItems];
  if (vec && i0 + kSumItems <= m) {  // 16-byte aligned: i0 is a multiple of 8
    const uint4 a = __ldg(reinterpret_cast<const uint4 *>(src + i0));
    const uint4 b = __ldg(reinterpret_cast<const uint4 *>(src + i0 + 4));
    r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w;
    r[4] = b.x; r[5] = b.y; r[6] = b.z; r[7] = b.w;
#pragma unroll
    for (int q = 0; q < kSumItems / 2; ++q) {
      const double2 d = __ldg(reinterpret_cast<const double2 *>(w + i0) + q);
      x[2 * q] = d.x;
      x[2 * q + 1] = d.y;
    }
  } else {
#pragma unroll
    for (int k = 0; k < kSumItems; ++k) {
      const bool ok = i0 + k < m;
      r[k] = ok ? __ldg(src + i0 + k) : kNoRow;
      x[k] = ok ? __ldg(w + i0 + k) : 0.0;
    }
  }
  // the rows of the entries on either side of the lane's run
  uint32_t prev = __shfl_up_sync(full, r[kSumItems - 1], 1);
  uint32_t next = __shfl_down_sync(full, r[0], 1);
  if (lane == 0) prev = T > 0 ? __ldg(src + T - 1) : kNoRow;
  if (lane == 31) next = T + kSumTile < m ? __ldg(src + T + kSumTile) : kNoRow;
  const bool first_cont = r[0] == prev;  // the first entry continues a row from the left
  double seg = 0.0, head = 0.0, tail = 0.0;
  bool head_done = false;  // the first piece continues from the left and ends its row here
  bool pass = false;       // the lane's last piece is its first and continues on both sides
#pragma unroll
  for (int k = 0; k < kSumItems; ++k) {
    const double v = clamp_weight(x[k]);
    const bool seg_first = k == 0 || r[k] != r[k - 1];
    seg = seg_first ? v : seg + v;
    const bool seg_end = k == kSumItems - 1 || r[k + 1] != r[k];
    if (seg_end) {
      const bool row_end = k < kSumItems - 1 || next != r[k];
      // this piece is the lane's first (from entry 0) and continues from the left
      bool from_left = first_cont;
#pragma unroll
      for (int j = 1; j <= k; ++j) from_left = from_left && r[j] == r[0];
      if (row_end && !from_left) {
        if (r[k] != kNoRow) rowsum[r[k]] = seg;
      } else if (row_end) {
        head = seg;
        head_done = true;
      } else {  // k is the lane's last entry: the piece continues to the right
        tail = seg;
        pass = from_left;
      }
    }
  }
  // segmented inclusive scan over the lanes: a lane passes the carry from its
  // left on only when its one piece continues on both sides
  double sc = tail;
  bool fl = lane == 0 || !pass;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double so = __shfl_up_sync(full, sc, o);
    const int fo = __shfl_up_sync(full, (int)fl, o);
    if (lane >= o) {
      if (!fl) sc = so + sc;
      fl = fl || fo;
    }
  }
  double carry = __shfl_up_sync(full, sc, 1);
  if (lane == 0) carry = 0.0;
  const bool tile_cont = __shfl_sync(full, (int)first_cont, 0) != 0;  // tile's first row began before it
  const uint32_t tile_row = __shfl_sync(full, r[0], 0);
  if (head_done) {
    const double tot = carry + head;
    if (tile_cont && r[0] == tile_row) thead[t] = tot;
    else rowsum[r[0]] = tot;
  }
  if (lane == 31 && r[kSumItems - 1] != kNoRow && next == r[kSumItems - 1]) tcarry[t] = sc;
}

// Rows 32*j .. 32*j+31 are one warp's: dmask word j is written whole.
__global__ void row_finish(int64_t n, const int64_t *__restrict__ rp, const double *__restrict__ tcarry,
                           const double *__restrict__ thead, double *__restrict__ rowsum,
                           uint32_t *__restrict__ dmask) {
  const int64_t words = (n + 31) / 32;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < words * 32;
       u += (int64_t)gridDim.x * blockDim.x) {  // uniform per warp: words * 32 rounds up
    bool dang = false;
    if (u < n) {
      const int64_t b = rp[u], e = rp[u + 1];
      double s = 0.0;
      if (e > b) {
        const int64_t t0 = b / kSumTile, t1 = (e - 1) / kSumTile;
        if (t0 == t1) {
          s = rowsum[u];
        } else {  // the tiles' pieces in order
          s = tcarry[t0];
          for (int64_t q = t0 + 1; q < t1; ++q) s += tcarry[q];
          s += thead[t1];
        }
      }
      dang = !(s > 0.0);
      rowsum[u] = dang ? 0.0 : 1.0 / s;
    }
    const unsigned bits = __ballot_sync(0xffffffffu, dang);
    if ((threadIdx.x & 31) == 0) dmask[u >> 5] = bits;
  }
}

__global__ void edge_weights(int64_t m, const double *__restrict__ w, const uint32_t *__restrict__ src,
                             const double *__restrict__ inv, uint2 *__restrict__ src_val) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const double wc = clamp_weight(w[i]);
    const uint32_t u = src[i];
    const float v = __double_as_longlong(wc) > 0 ? (float)(wc * inv[u]) : 0.0f;
    src_val[i] = make_uint2(u, __float_as_uint(v));
  }
}

// rp[v] = first position i of the sorted destination keys K with K[i] >= v
// (v = 0..n): a binary search per node, so that no thread writes a long run
// of rows without in-edges (the searches of neighbouring nodes share their
// first probes in cache).
__global__ void rp_from_sorted(const uint32_t *K, int64_t m, int64_t n, int64_t *rp) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v <= n;
       v += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = m;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if ((int64_t)__ldg(&K[mid]) < v) lo = mid + 1;
      else hi = mid;
    }
    rp[v] = lo;
  }
}

__global__ void max_indeg(const int64_t *rp, int64_t n, unsigned *out) {
  unsigned best = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x)
    best = max(best, (unsigned)(rp[v + 1] - rp[v]));
  best = __reduce_max_sync(0xffffffffu, best);
  if ((threadIdx.x & 31) == 0) atomicMax(out, best);
}

__global__ void node_sort_keys(const int64_t *rp, int64_t n, const unsigned *maxdeg,
                               uint32_t *keys, uint32_t *vals) {
  const unsigned md = *maxdeg;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    keys[v] = md - (unsigned)(rp[v + 1] - rp[v]);
    vals[v] = (uint32_t)v;
  }
}

// Row i of the relabelled graph is node perm[i] = sorted_vals[i].
__global__ void permute_nodes(const uint32_t *sorted_keys, const uint32_t *sorted_vals, int64_t n,
                              const unsigned *maxdeg, int32_t *perm, int32_t *inv_perm,
                              int64_t *new_deg, const float *deg_old, float *deg_new) {
  const unsigned md = *maxdeg;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t old = sorted_vals[i];
    perm[i] = (int32_t)old;
    inv_perm[old] = (int32_t)i;
    new_deg[i] = (int64_t)(md - sorted_keys[i]);
    deg_new[i] = deg_old[old];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) new_deg[n] = 0;
}

__global__ void permute_dmask(const int32_t *perm, int64_t n, const uint32_t *old_mask,
                              uint32_t *new_mask) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < n;
  unsigned bit = 0;
  if (valid) {
    const int32_t o = perm[i];
    bit = (old_mask[o >> 5] >> (o & 31)) & 1u;
  }
  const unsigned word = __ballot_sync(0xffffffffu, bit);
  if ((threadIdx.x & 31) == 0 && i < n) new_mask[i >> 5] = word;
}

// Sorted position i holds edge O[i] into node K[i]; it lands in relabelled
// row inv_perm[K[i]] at the same offset within the row.
__global__ void scatter_edges(const uint32_t *K, const uint32_t *O, int64_t m, const int64_t *rp_old,
                              const int32_t *inv_perm, const int64_t *rp_new, const uint32_t *src,
                              const uint2 *src_val, int32_t *in_col, float *in_val) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t v = K[i];
    const int64_t pos = rp_new[inv_perm[v]] + (i - rp_old[v]);
    const uint32_t e = O[i];
    if (src_val) {  // weighted: source and weight in one load
      const uint2 sv = src_val[e];
      in_col[pos] = inv_perm[sv.x];
      in_val[pos] = __uint_as_float(sv.y);
    } else {
      in_col[pos] = inv_perm[src[e]];
    }
  }
}

__global__ void pad_degrees(int64_t *deg, int64_t n, int align) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    deg[i] = (deg[i] + align - 1) / align * align;
}

// Slots of the relabelled in-CSR that no edge fills: the padding of row i
// (md - sorted_keys[i] edges in a run rounded up to kRowAlign slots) and the
// kTailSlots slots past the last row, read by vector loads: source n (whose
// gathered value is 0) and weight 0.
constexpr int64_t kTailSlots = 64;

__global__ void pad_slots(const uint32_t *sorted_keys, const unsigned *maxdeg, const int64_t *in_rp, int64_t n,
                          int32_t *in_col, float *in_val) {
  const unsigned md = *maxdeg;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n + kTailSlots;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t b, e;
    if (i < n) {
      b = in_rp[i] + (int64_t)(md - sorted_keys[i]);
      e = in_rp[i + 1];
    } else {
      b = in_rp[n] + (i - n);
      e = b + 1;
    }
    for (int64_t j = b; j < e; ++j) {
      in_col[j] = (int32_t)n;
      if (in_val) in_val[j] = 0.0f;
    }
  }
}

// out[j] = number of relabelled rows with in-degree >= thr[j] (degrees are
// non-increasing along the rows: maxdeg - sorted_keys[i]).
__global__ void count_ge(const uint32_t *sorted_keys, int64_t n, const unsigned *maxdeg,
                         const int64_t *thr, int nthr, int64_t *out) {
  const int j = threadIdx.x;
  if (j >= nthr) return;
  const unsigned md = *maxdeg;
  int64_t lo = 0, hi = n;  // first row with degree < thr
  while (lo < hi) {
    const int64_t mid = (lo + hi) / 2;
    if ((int64_t)(md - sorted_keys[mid]) >= thr[j]) lo = mid + 1;
    else hi = mid;
  }
  out[j] = lo;
}

__global__ void hub_chunks(const int64_t *rp, int32_t n_hub, int64_t *nch) {
  for (int32_t h = blockIdx.x * blockDim.x + threadIdx.x; h <= n_hub; h += gridDim.x * blockDim.x)
    nch[h] = h < n_hub ? ceil_div<int64_t>(rp[h + 1] - rp[h], kHubChunk) : 0;
}

__global__ void hub_fill(const int64_t *first64, int32_t n_hub, int32_t *first, int32_t *task_row) {
  for (int32_t h = blockIdx.x * blockDim.x + threadIdx.x; h <= n_hub; h += gridDim.x * blockDim.x) {
    first[h] = (int32_t)first64[h];
    if (h < n_hub)
      for (int64_t t = first64[h]; t < first64[h + 1]; ++t) task_row[t] = h;
  }
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

// ---- edge-list ingestion (a petgraph Graph's raw edges, in edge order) ----

// keys[i] = src[m - 1 - i] (the edge list reversed), with the range checks
__global__ void reversed_sources(const int32_t *src, const int32_t *dst, int64_t m, int64_t n, uint32_t *keys,
                                 int *bad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = m - 1 - i;
    const int32_t a = src[e], b = dst[e];
    if (a < 0 || a >= n || b < 0 || b >= n) *bad = 1;
    keys[i] = (uint32_t)min(max(a, 0), (int32_t)(n - 1));
  }
}

// out-CSR entry k: the edge at position vals[k] of the reversed list
__global__ void edges_gather(const uint32_t *vals, const int32_t *dst, const double *w, int64_t m, int32_t *col,
                             double *wraw, uint32_t *colkey) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = m - 1 - (int64_t)vals[k];
    col[k] = dst[e];
    colkey[k] = (uint32_t)dst[e];
    if (w) wraw[k] = w[e];
  }
}

// keys2[i] = source row of out-CSR entry pos[i]
__global__ void row_of_positions(const uint32_t *rows, const uint32_t *pos, int64_t m, uint32_t *keys2) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
    keys2[i] = rows[pos[i]];
}

// Entries ordered by (row, target), ties in row order: start[i] = 1 where a
// (row, target) run begins.
__global__ void run_starts(const uint32_t *rows, const uint32_t *pos, const int32_t *col, int64_t m, int64_t *start) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t p = pos[i];
    bool st = i == 0;
    if (!st) {
      const uint32_t q = pos[i - 1];
      st = rows[p] != rows[q] || col[p] != col[q];
    }
    start[i] = st ? 1 : 0;
  }
}

// find_edge's weight: every entry of a run gets the weight of the run's
// first entry in row order (petgraph's walk meets the newest edge first)
__global__ void run_weights(const int64_t *run_excl, const int64_t *start, const uint32_t *pos, const double *wraw,
                            int64_t m, double *first_w, double *wout, int pass) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t run = run_excl[i] + start[i] - 1;
    if (pass == 0) {
      if (start[i]) first_w[run] = wraw[pos[i]];
    } else {
      wout[pos[i]] = first_w[run];
    }
  }
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

void graph_free_device(Graph &g) {
  cudaFree(g.in_rp); cudaFree(g.in_col); cudaFree(g.in_val); cudaFree(g.deg);
  cudaFree(g.dmask_w); cudaFree(g.perm); cudaFree(g.hub_first); cudaFree(g.hub_task_row);
  cudaFree(g.out_rp); cudaFree(g.out_col);
  workspace_free(g.ws);
  batch_free(g);
  g.in_rp = nullptr; g.in_col = nullptr; g.in_val = nullptr; g.deg = nullptr;
  g.dmask_w = nullptr; g.perm = nullptr; g.hub_first = nullptr; g.hub_task_row = nullptr;
  g.out_rp = nullptr; g.out_col = nullptr;
}

Status graph_build_from_out_csr_device(Ctx *ctx, Graph *g, const int64_t *d_out_rp,
                                       const int32_t *d_out_col, const double *d_w,
                                       cudaEvent_t w_ready) {
  cudaStream_t s = ctx->stream;
  const int64_t n = g->n, m = g->m;
  g->weighted = d_w != nullptr;
  Status st;
  uint32_t *src = nullptr, *keys = nullptr, *vals = nullptr, *keys2 = nullptr, *vals2 = nullptr;
  uint32_t *nk = nullptr, *nv = nullptr, *nk2 = nullptr, *nv2 = nullptr, *dmask_old = nullptr;
  float *deg_old = nullptr;
  uint2 *src_val = nullptr;
  int64_t *rp_old = nullptr, *new_deg = nullptr, *small = nullptr;
  int32_t *inv_perm = nullptr;
  unsigned *maxdeg = nullptr;
  uint32_t *bigrows = nullptr;
  double *rowsum = nullptr, *tcarry = nullptr, *thead = nullptr;
  // weight passes queued on the copy stream (the main stream waits for them
  // before any buffer they use is freed)
  bool copy_side = false;
  auto cleanup = [&]() {
    if (copy_side) cudaStreamWaitEvent(s, ctx->build_ev[1], 0);
    free_async(src, s); free_async(keys, s); free_async(vals, s); free_async(keys2, s);
    free_async(vals2, s); free_async(nk, s); free_async(nv, s); free_async(nk2, s);
    free_async(nv2, s); free_async(dmask_old, s); free_async(src_val, s); free_async(deg_old, s);
    free_async(rp_old, s); free_async(new_deg, s); free_async(small, s); free_async(inv_perm, s);
    free_async(maxdeg, s); free_async(bigrows, s); free_async(rowsum, s);
    free_async(tcarry, s); free_async(thead, s);
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
#define BUILD_ST(expr)                       \
  do {                                       \
    st = (expr);                             \
    if (st.code != GOPS_OK) { cleanup(); return st; } \
  } while (0)
  const size_t mm = (size_t)std::max<int64_t>(m, 1) + 64;  // padded edge arrays
  const size_t nn = (size_t)std::max<int64_t>(n, 1);
  const size_t nwords = (size_t)(n / 32 + 1);
  BUILD_TRY(dev_malloc_async(&g->in_rp, sizeof(int64_t) * (n + 1), s));
  BUILD_TRY(dev_malloc_async(&g->deg, sizeof(float) * nn, s));
  BUILD_TRY(dev_malloc_async(&g->perm, sizeof(int32_t) * nn, s));
  BUILD_TRY(dev_malloc_async((void **)&deg_old, sizeof(float) * nn, s));
  if (g->weighted) {
    BUILD_TRY(dev_malloc_async(&g->dmask_w, sizeof(uint32_t) * nwords, s));
    BUILD_TRY(cudaMemsetAsync(g->dmask_w, 0, sizeof(uint32_t) * nwords, s));
    BUILD_TRY(dev_malloc_async((void **)&dmask_old, sizeof(uint32_t) * nwords, s));
    BUILD_TRY(cudaMemsetAsync(dmask_old, 0, sizeof(uint32_t) * nwords, s));
    BUILD_TRY(dev_malloc_async((void **)&src_val, sizeof(uint2) * mm, s));
    BUILD_TRY(dev_malloc_async((void **)&rowsum, sizeof(double) * nn, s));
  }
  // K1: stable sort of edge ids by destination
  BUILD_TRY(dev_malloc_async((void **)&keys, sizeof(uint32_t) * mm, s));
  BUILD_TRY(dev_malloc_async((void **)&vals, sizeof(uint32_t) * mm, s));
  BUILD_TRY(dev_malloc_async((void **)&keys2, sizeof(uint32_t) * mm, s));
  BUILD_TRY(dev_malloc_async((void **)&vals2, sizeof(uint32_t) * mm, s));
  uint32_t *K = keys, *O = vals;
  if (m > 0) {
    bool alt = false;  // keys: the destination ids; values: the edge ids
    BUILD_ST(radix_sort_index_u32(reinterpret_cast<const uint32_t *>(d_out_col), keys, vals, keys2, vals2, m,
                                  bits_for(n), &alt, s));
    if (alt) { K = keys2; O = vals2; }
  }
  BUILD_TRY(dev_malloc_async((void **)&src, sizeof(uint32_t) * mm, s));
  if (n > 0) {  // structure pass: no weights read
    // rows longer than kRowBig: at most m / (kRowBig + 1) of them
    const int64_t nbig_cap = std::min<int64_t>(n, m / (kRowBig + 1)) + 1;
    BUILD_TRY(dev_malloc_async((void **)&bigrows, sizeof(uint32_t) * nbig_cap, s));
    BUILD_TRY(cudaMemsetAsync(bigrows, 0, sizeof(uint32_t), s));
    out_rows<<<grid_for(n, 256 / kRowLanes), 256, 0, s>>>(n, d_out_rp, src, deg_old, bigrows);
    out_rows_big<<<ctx->num_sms * 4, 256, 0, s>>>(d_out_rp, src, deg_old, bigrows);
    BUILD_TRY(cudaGetLastError());
  }
  // the weight passes' per-tile pieces of rows that cross a tile's ends
  const int64_t wtiles = ceil_div<int64_t>(m, kSumTile);
  if (d_w && m > 0) {
    BUILD_TRY(dev_malloc_async((void **)&tcarry, sizeof(double) * wtiles, s));
    BUILD_TRY(dev_malloc_async((void **)&thead, sizeof(double) * wtiles, s));
  }
  auto weight_passes = [&](cudaStream_t st) {
    if (m > 0) {
      const int vec = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(d_w)) & 15) == 0;
      row_sums_tiles<<<(unsigned)ceil_div<int64_t>(wtiles, 8), 256, 0, st>>>(m, src, d_w, vec, rowsum, tcarry, thead);
    }
    row_finish<<<blocks_for(n, 256, ctx->num_sms * 8), 256, 0, st>>>(n, d_out_rp, tcarry, thead, rowsum, dmask_old);
    if (m > 0) edge_weights<<<blocks_for(m, 256, ctx->num_sms * 8), 256, 0, st>>>(m, d_w, src, rowsum, src_val);
  };
  // The weight passes need the weights, the structure pass and nothing of
  // the relabelling: with the weights arriving on the copy stream they run
  // there as soon as both are done, beside the main stream's relabelling.
  if (w_ready && d_w && n > 0) {
    cudaStream_t cs = ctx->copy_stream;
    BUILD_TRY(cudaEventRecord(ctx->build_ev[0], s));
    BUILD_TRY(cudaStreamWaitEvent(cs, ctx->build_ev[0], 0));
    BUILD_TRY(cudaStreamWaitEvent(cs, w_ready, 0));
    copy_side = true;
    weight_passes(cs);
    BUILD_TRY(cudaGetLastError());
    BUILD_TRY(cudaEventRecord(ctx->build_ev[1], cs));
  }
  BUILD_TRY(dev_malloc_async((void **)&rp_old, sizeof(int64_t) * (n + 1), s));
  rp_from_sorted<<<grid_for(n + 1, 256), 256, 0, s>>>(K, m, n, rp_old);
  BUILD_TRY(cudaGetLastError());
  // K2: relabel by in-degree, descending (stable: ties keep id order)
  BUILD_TRY(dev_malloc_async((void **)&maxdeg, sizeof(unsigned), s));
  BUILD_TRY(cudaMemsetAsync(maxdeg, 0, sizeof(unsigned), s));
  BUILD_TRY(dev_malloc_async((void **)&nk, sizeof(uint32_t) * nn, s));
  BUILD_TRY(dev_malloc_async((void **)&nv, sizeof(uint32_t) * nn, s));
  BUILD_TRY(dev_malloc_async((void **)&nk2, sizeof(uint32_t) * nn, s));
  BUILD_TRY(dev_malloc_async((void **)&nv2, sizeof(uint32_t) * nn, s));
  BUILD_TRY(dev_malloc_async((void **)&inv_perm, sizeof(int32_t) * nn, s));
  BUILD_TRY(dev_malloc_async((void **)&new_deg, sizeof(int64_t) * (n + 1), s));
  unsigned md = 0;
  uint32_t *SK = nk, *SV = nv;
  if (n > 0) {
    max_indeg<<<blocks_for(n, 256, ctx->num_sms * 4), 256, 0, s>>>(rp_old, n, maxdeg);
    node_sort_keys<<<grid_for(n, 256), 256, 0, s>>>(rp_old, n, maxdeg, nk, nv);
    BUILD_TRY(cudaGetLastError());
    BUILD_TRY(cudaMemcpyAsync(&md, maxdeg, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    BUILD_TRY(cudaStreamSynchronize(s));
    bool alt = false;
    BUILD_ST(radix_sort_pairs_u32(nk, nv, nk2, nv2, n, bits_for((int64_t)md + 1), &alt, s));
    if (alt) { SK = nk2; SV = nv2; }
    permute_nodes<<<grid_for(n, 256), 256, 0, s>>>(SK, SV, n, maxdeg, g->perm, inv_perm, new_deg,
                                                   deg_old, g->deg);
    BUILD_TRY(cudaGetLastError());
  } else {
    BUILD_TRY(cudaMemsetAsync(new_deg, 0, sizeof(int64_t), s));
  }
  if (kRowAlign > 1 && n > 0) {
    pad_degrees<<<grid_for(n, 256), 256, 0, s>>>(new_deg, n, kRowAlign);
    BUILD_TRY(cudaGetLastError());
  }
  BUILD_ST(exclusive_scan_i64(new_deg, g->in_rp, n + 1, s));
  int64_t m_stored = 0;
  BUILD_TRY(cudaMemcpyAsync(&m_stored, g->in_rp + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  BUILD_TRY(cudaStreamSynchronize(s));
  g->m_stored = m_stored;
  const size_t ms = (size_t)m_stored + kTailSlots;  // vector loads past the end
  BUILD_TRY(dev_malloc_async(&g->in_col, sizeof(int32_t) * ms, s));
  if (g->weighted) BUILD_TRY(dev_malloc_async(&g->in_val, sizeof(float) * ms, s));
  // the slots that no edge fills (the scatter writes the others)
  pad_slots<<<grid_for(n + kTailSlots, 256), 256, 0, s>>>(SK, maxdeg, g->in_rp, n, g->in_col, g->in_val);
  BUILD_TRY(cudaGetLastError());
  // the weights: everything above ran while they were being copied
  if (copy_side) {
    BUILD_TRY(cudaStreamWaitEvent(s, ctx->build_ev[1], 0));
  } else {
    if (w_ready) BUILD_TRY(cudaStreamWaitEvent(s, w_ready, 0));
    if (d_w && n > 0) {
      weight_passes(s);
    }
  }
  if (d_w && n > 0) {
    permute_dmask<<<(unsigned)ceil_div<int64_t>(n, 256), 256, 0, s>>>(g->perm, n, dmask_old, g->dmask_w);
    BUILD_TRY(cudaGetLastError());
  }
  if (m > 0) {
    scatter_edges<<<grid_for(m, 256), 256, 0, s>>>(K, O, m, rp_old, inv_perm, g->in_rp, src, src_val,
                                                   g->in_col, g->in_val);
    BUILD_TRY(cudaGetLastError());
  }
  // plan: degree classes over the (non-increasing) relabelled degrees
  const int L = kLaneEdges;
  const int64_t thr_h[7] = {kHubThreshold + 1, 32 * L, 16 * L, 8 * L, 4 * L, 2 * L, 0};
  int64_t cnt_h[7] = {0, 0, 0, 0, 0, 0, 0};
  BUILD_TRY(dev_malloc_async((void **)&small, sizeof(int64_t) * 16, s));
  if (n > 0) {
    BUILD_TRY(cudaMemcpyAsync(small, thr_h, sizeof(thr_h), cudaMemcpyHostToDevice, s));
    count_ge<<<1, 32, 0, s>>>(SK, n, maxdeg, small, 7, small + 8);
    BUILD_TRY(cudaGetLastError());
    BUILD_TRY(cudaMemcpyAsync(cnt_h, small + 8, sizeof(cnt_h), cudaMemcpyDeviceToHost, s));
    BUILD_TRY(cudaStreamSynchronize(s));
  }
  Plan &pl = g->plan;
  pl = Plan{};
  pl.n_hub = (int32_t)cnt_h[0];
  const int sws[6] = {32, 16, 8, 4, 2, 1};
  int64_t row = pl.n_hub, task = 0;
  for (int c = 0; c < 6; ++c) {
    const int64_t end = c == 5 ? n : std::max<int64_t>(row, cnt_h[c + 1]);
    if (end > row) {
      Segment &sg = pl.segs[pl.n_segs++];
      sg.row_begin = (int32_t)row;
      sg.row_end = (int32_t)end;
      sg.sw = sws[c];
      sg.task_begin = (int32_t)task;  // relative to the first segment task
      task += ceil_div<int64_t>((end - row) * sws[c], 32 * kRowsPerLane);
      row = end;
    }
  }
  // hub tasks
  if (pl.n_hub > 0) {
    int64_t *nch = nullptr;
    BUILD_TRY(dev_malloc_async((void **)&nch, sizeof(int64_t) * (pl.n_hub + 1), s));
    hub_chunks<<<grid_for(pl.n_hub + 1, 256), 256, 0, s>>>(g->in_rp, pl.n_hub, nch);
    Status s2 = exclusive_scan_i64(nch, nch, pl.n_hub + 1, s);
    int64_t nht = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && s2.code == GOPS_OK)
      e = cudaMemcpyAsync(&nht, nch + pl.n_hub, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    const bool ok = e == cudaSuccess && s2.code == GOPS_OK;  // nch holds offsets only then
    if (ok) e = dev_malloc_async(&g->hub_first, sizeof(int32_t) * (pl.n_hub + 1), s);
    if (ok && e == cudaSuccess) e = dev_malloc_async(&g->hub_task_row, sizeof(int32_t) * std::max<int64_t>(nht, 1), s);
    if (ok && e == cudaSuccess) {
      hub_fill<<<grid_for(pl.n_hub + 1, 256), 256, 0, s>>>(nch, pl.n_hub, g->hub_first, g->hub_task_row);
      e = cudaGetLastError();
    }
    free_async(nch, s);
    if (s2.code != GOPS_OK) { cleanup(); return s2; }
    BUILD_TRY(e);
    pl.n_hub_tasks = (int32_t)nht;
  }
  for (int i = 0; i < pl.n_segs; ++i) pl.segs[i].task_begin += pl.n_hub_tasks;
  if (task + pl.n_hub_tasks >= INT32_MAX) { cleanup(); return Status{GOPS_ERR_INVALID, "graph too large"}; }
  pl.n_tasks = (int32_t)(task + pl.n_hub_tasks);
  BUILD_TRY(cudaStreamSynchronize(s));
  cleanup();
  return Status::ok();
#undef BUILD_TRY
#undef BUILD_ST
}

// Dense AdjacencyMatrix -> device out-CSR -> the build above.
Status dense_to_out_csr_device(Ctx *ctx, int64_t n, const double *d_M, int64_t **d_rp,
                               int32_t **d_col, double **d_w, int64_t *m_out) {
  cudaStream_t s = ctx->stream;
  *d_rp = nullptr; *d_col = nullptr; *d_w = nullptr;
  GOPS_CUDA_TRY(dev_malloc_async((void **)d_rp, sizeof(int64_t) * (n + 1), s));
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
  GOPS_CUDA_TRY(dev_malloc_async((void **)d_col, sizeof(int32_t) * std::max<int64_t>(m, 1), s));
  GOPS_CUDA_TRY(dev_malloc_async((void **)d_w, sizeof(double) * std::max<int64_t>(m, 1), s));
  if (n > 0 && m > 0) {
    dense_rows<<<(unsigned)ceil_div<int64_t>(n, 8), 256, 0, s>>>(n, d_M, nullptr, *d_rp, *d_col,
                                                                 *d_w);
    GOPS_CUDA_TRY(cudaGetLastError());
  }
  return Status::ok();
}

// A petgraph Graph<_, f64, Directed>'s raw edge list (edge e: src[e] ->
// dst[e], weight w[e], in edge-index order) -> the out-CSR its adapter
// exposes (src/graph.rs:144-212): row u lists the targets of u's outgoing
// edges newest first (petgraph walks a node's edge list from its last
// added edge; parallel edges are repeated), and with weights, every entry
// u -> v carries the weight find_edge(u, v) returns, that of the newest
// u -> v edge.  A stable radix sort of the reversed edge list by source gives
// the rows; a stable sort of the entries by (source, target) groups the
// parallel edges, and each group takes the weight of its first entry.
Status edges_to_out_csr_device(Ctx *ctx, int64_t n, int64_t m, const int32_t *d_src, const int32_t *d_dst,
                               const double *d_w, int64_t **d_rp, int32_t **d_col, double **d_wout) {
  cudaStream_t s = ctx->stream;
  *d_rp = nullptr; *d_col = nullptr; *d_wout = nullptr;
  const int64_t mm = std::max<int64_t>(m, 1);
  uint32_t *kin = nullptr, *k1 = nullptr, *v1 = nullptr, *k2 = nullptr, *v2 = nullptr, *colkey = nullptr;
  double *wraw = nullptr, *first_w = nullptr;
  int64_t *start = nullptr, *excl = nullptr;
  int *bad = nullptr;
  auto cleanup = [&]() {
    free_async(kin, s); free_async(k1, s); free_async(v1, s); free_async(k2, s); free_async(v2, s);
    free_async(colkey, s); free_async(wraw, s); free_async(first_w, s); free_async(start, s); free_async(excl, s);
    free_async(bad, s);
  };
  auto fail_all = [&](Status st) {
    cleanup();
    free_async(*d_rp, s); free_async(*d_col, s); free_async(*d_wout, s);
    *d_rp = nullptr; *d_col = nullptr; *d_wout = nullptr;
    return st;
  };
#define EDGE_TRY(expr)                                                                           \
  do {                                                                                           \
    cudaError_t _e = (expr);                                                                     \
    if (_e != cudaSuccess)                                                                       \
      return fail_all(Status{_e == cudaErrorMemoryAllocation ? GOPS_ERR_OOM : GOPS_ERR_CUDA,      \
                             std::string("edge list: ") + cudaGetErrorString(_e)});              \
  } while (0)
#define EDGE_ST(expr)                          \
  do {                                         \
    Status _s = (expr);                        \
    if (_s.code != GOPS_OK) return fail_all(_s); \
  } while (0)
  EDGE_TRY(dev_malloc_async((void **)d_rp, sizeof(int64_t) * (n + 1), s));
  EDGE_TRY(dev_malloc_async((void **)d_col, sizeof(int32_t) * mm, s));
  EDGE_TRY(dev_malloc_async((void **)&kin, sizeof(uint32_t) * mm, s));
  EDGE_TRY(dev_malloc_async((void **)&k1, sizeof(uint32_t) * mm, s));
  EDGE_TRY(dev_malloc_async((void **)&v1, sizeof(uint32_t) * mm, s));
  EDGE_TRY(dev_malloc_async((void **)&k2, sizeof(uint32_t) * mm, s));
  EDGE_TRY(dev_malloc_async((void **)&v2, sizeof(uint32_t) * mm, s));
  EDGE_TRY(dev_malloc_async((void **)&colkey, sizeof(uint32_t) * mm, s));
  EDGE_TRY(dev_malloc_async((void **)&bad, sizeof(int), s));
  EDGE_TRY(cudaMemsetAsync(bad, 0, sizeof(int), s));
  if (m > 0) {
    reversed_sources<<<grid_for(m, 256), 256, 0, s>>>(d_src, d_dst, m, n, kin, bad);
    EDGE_TRY(cudaGetLastError());
  }
  int hbad = 0;
  EDGE_TRY(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  EDGE_TRY(cudaStreamSynchronize(s));
  if (hbad) return fail_all(Status{GOPS_ERR_INVALID, "edge endpoint out of range"});
  // rows: sources ascending, each source's edges newest first
  bool alt = false;
  const int bits = std::max(1, bits_for(n));
  EDGE_ST(radix_sort_index_u32(kin, k1, v1, k2, v2, m, bits, &alt, s));
  const uint32_t *rows = alt ? k2 : k1;
  const uint32_t *pos_rev = alt ? v2 : v1;
  rp_from_sorted<<<grid_for(n + 1, 256), 256, 0, s>>>(rows, m, n, *d_rp);
  EDGE_TRY(cudaGetLastError());
  if (d_w) {
    EDGE_TRY(dev_malloc_async((void **)&wraw, sizeof(double) * mm, s));
    EDGE_TRY(dev_malloc_async((void **)d_wout, sizeof(double) * mm, s));
  }
  if (m > 0) {
    edges_gather<<<grid_for(m, 256), 256, 0, s>>>(pos_rev, d_dst, d_w, m, *d_col, wraw, colkey);
    EDGE_TRY(cudaGetLastError());
  }
  if (d_w && m > 0) {
    // the row keys move out of the sort buffers, which the next sorts reuse
    uint32_t *rowk = kin;
    EDGE_TRY(cudaMemcpyAsync(rowk, rows, sizeof(uint32_t) * m, cudaMemcpyDeviceToDevice, s));
    // entries by target (stable), then by row (stable): (row, target) order, ties in row order
    EDGE_ST(radix_sort_index_u32(colkey, k1, v1, k2, v2, m, bits, &alt, s));
    const uint32_t *pos_t = alt ? v2 : v1;
    uint32_t *kb = alt ? k1 : k2;  // a key buffer not holding the result
    uint32_t *keys2 = colkey;                           // colkey is no longer needed
    row_of_positions<<<grid_for(m, 256), 256, 0, s>>>(rowk, pos_t, m, keys2);
    EDGE_TRY(cudaGetLastError());
    uint32_t *vin = kb;
    EDGE_TRY(cudaMemcpyAsync(vin, pos_t, sizeof(uint32_t) * m, cudaMemcpyDeviceToDevice, s));
    uint32_t *kk1 = nullptr, *vv1 = nullptr;
    EDGE_TRY(dev_malloc_async((void **)&kk1, sizeof(uint32_t) * mm, s));
    EDGE_TRY(dev_malloc_async((void **)&vv1, sizeof(uint32_t) * mm, s));
    bool alt2 = false;
    Status st2 = radix_sort_pairs_u32(keys2, vin, kk1, vv1, m, bits, &alt2, s);
    const uint32_t *pos = alt2 ? vv1 : vin;
    EDGE_TRY(dev_malloc_async((void **)&start, sizeof(int64_t) * (m + 1), s));
    EDGE_TRY(dev_malloc_async((void **)&excl, sizeof(int64_t) * (m + 1), s));
    EDGE_TRY(dev_malloc_async((void **)&first_w, sizeof(double) * mm, s));
    if (st2.code == GOPS_OK) {
      run_starts<<<grid_for(m, 256), 256, 0, s>>>(rowk, pos, *d_col, m, start);
      st2 = cudaGetLastError() == cudaSuccess ? Status::ok() : Status{GOPS_ERR_CUDA, "run_starts"};
    }
    if (st2.code == GOPS_OK) st2 = exclusive_scan_i64(start, excl, m, s);
    if (st2.code == GOPS_OK) {
      run_weights<<<grid_for(m, 256), 256, 0, s>>>(excl, start, pos, wraw, m, first_w, *d_wout, 0);
      run_weights<<<grid_for(m, 256), 256, 0, s>>>(excl, start, pos, wraw, m, first_w, *d_wout, 1);
      st2 = cudaGetLastError() == cudaSuccess ? Status::ok() : Status{GOPS_ERR_CUDA, "run_weights"};
    }
    free_async(kk1, s);
    free_async(vv1, s);
    EDGE_ST(st2);
  }
  EDGE_TRY(cudaStreamSynchronize(s));
  cleanup();
  return Status::ok();
#undef EDGE_TRY
#undef EDGE_ST
}

}  // namespace gops
