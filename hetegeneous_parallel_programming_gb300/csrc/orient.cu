// Degree-ordered orientation on the device.
//
// Rule (reference successful_push_pull/graph.cc:265-266): keep u->v iff
// deg(v) > deg(u) or (deg(v) == deg(u) and v > u).  That is exactly
// rank(u) < rank(v) for rank = position in ascending (degree, id) order, so
// the engine sorts the n keys (deg << B | id), keeps an entry iff the rank
// grows, compacts kept entries in input order (which is the reference's
// output order, graph.cc:279-290) and radix-sorts them by (rank(u), rank(v))
// into the relabelled DAG the count kernels read.
#include "engine.cuh"

namespace tc {

constexpr int OR_THREADS = 256;
constexpr int OR_PER = ENTRY_TILE / OR_THREADS;  // 8 entries per thread per tile
// Every relabelled entry's row (nsrc): 1: the placement writes it next to
// its column (a second scattered store per entry); 2: the row sorts write it,
// coalesced, for the rows they visit (rows of one entry included); 0: a
// streaming pass derives it from the relabelled row pointers afterwards
#ifndef TC_PLACE_SRC
#define TC_PLACE_SRC 2
#endif
constexpr bool PLACE_SRC = TC_PLACE_SRC == 1;
constexpr bool SORT_SRC = TC_PLACE_SRC == 2;
// 1: the placement reads each row's destination base from rowbase_kernel's
// per-vertex array; 0: it gathers nrowptr[rank u] and orowptr[u] itself
#ifndef TC_PLACE_ROWBASE
#define TC_PLACE_ROWBASE 1
#endif
constexpr bool PLACE_ROWBASE = TC_PLACE_ROWBASE != 0;

// src[b .. b + L) = r by threads tid, tid + nt, ... (the row sorts' nsrc writes)
__device__ __forceinline__ void put_row_src(int32_t *__restrict__ src, int64_t b, int L, int32_t r, int tid, int nt) {
  if (src)
    for (int k = tid; k < L; k += nt) src[b + k] = r;
}
// 1: rows of <= 32 entries are sorted by a warp per 32 consecutive rows
#ifndef TC_SEG_WARP_CHUNK
#define TC_SEG_WARP_CHUNK 1
#endif
constexpr bool SEG_WARP_CHUNK = TC_SEG_WARP_CHUNK != 0;
// 1: rows of 33..256 entries are sorted with their keys in registers
// (seg_sort_warpreg_kernel); 0: in a warp's shared-memory slice
#ifndef TC_SEG_WARP_REG
#define TC_SEG_WARP_REG 1
#endif
constexpr bool SEG_WARP_REG = TC_SEG_WARP_REG != 0;
// 1: rows of 257..4096 entries whose ids span <= 32768 values are sorted
// through a warp's bitmap (seg_sort_warpbits_kernel) before the block sort
#ifndef TC_SEG_WARP_BITS
#define TC_SEG_WARP_BITS 1
#endif
constexpr bool SEG_WARP_BITS = TC_SEG_WARP_BITS != 0;

void orient_geometry(const tc_ctx *ctx, int64_t nnz, int pieces, int *G, int64_t *chunk) {
  int64_t tiles = (nnz + ENTRY_TILE - 1) / ENTRY_TILE;
  // blocks of 256 per SM in the entry-chunk geometry (6 are resident at once)
  int64_t g = (int64_t)ctx->num_sms * ctx->orient_blocks_per_sm * pieces;
  if (g > tiles) g = tiles;
  if (g < 1) g = 1;
  *chunk = ((tiles + g - 1) / g) * ENTRY_TILE;
  if (*chunk < ENTRY_TILE) *chunk = ENTRY_TILE;
  *G = (int)((nnz + *chunk - 1) / *chunk);
  if (*G < 1) *G = 1;
}

static inline int vertex_bits(int64_t n) { return bit_width_u64(n > 1 ? (uint64_t)(n - 1) : 1); }

// ---- validation -------------------------------------------------------------------

__global__ void validate_rowptr_kernel(const int64_t *__restrict__ rowptr, int64_t n, int64_t nnz,
                                       unsigned *flags) {
  unsigned f = 0;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u <= n; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = rowptr[u];
    if (u == 0 && a != 0) f |= VF_ROWPTR_ENDS;
    if (u == n && a != nnz) f |= VF_ROWPTR_ENDS;
    if (u < n && rowptr[u + 1] < a) f |= VF_ROWPTR_ORDER;
    if (a < 0 || a > nnz) f |= VF_ROWPTR_ENDS;
  }
  f = __reduce_or_sync(TC_FULL_MASK, f);
  if ((threadIdx.x & 31) == 0 && f) atomicOr(flags, f);
}

__global__ void __launch_bounds__(OR_THREADS) validate_col_kernel(const int64_t *__restrict__ rowptr,
                                                                 const int32_t *__restrict__ col, int64_t n,
                                                                 int64_t nnz, int simple, unsigned *flags) {
  __shared__ int rows[row_slots<ENTRY_TILE>()];
  __shared__ int scan_tmp[32];
  unsigned f = 0;
  const int64_t tiles = (nnz + ENTRY_TILE - 1) / ENTRY_TILE;
  for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int64_t t0 = t * ENTRY_TILE, t1 = min(nnz, t0 + ENTRY_TILE);
    int64_t hint = -1;  // tiles of one block are not contiguous here
    if (simple) expand_rows<ENTRY_TILE>(rowptr, n, t0, t1, rows, scan_tmp, hint);
#pragma unroll
    for (int k = 0; k < OR_PER; ++k) {
      const int64_t e = t0 + k * OR_THREADS + threadIdx.x;
      if (e >= t1) continue;
      const int32_t v = col[e];
      if (v < 0 || (int64_t)v >= n) { f |= VF_ID_RANGE; continue; }
      if (simple) {
        const int u = rows[rslot((int)(e - t0))];
        if (u == v) f |= VF_SELF_LOOP;
        if (u >= 0 && u < n && e > 0 && e > rowptr[u] && col[e - 1] >= v) f |= VF_UNSORTED;
      }
    }
    __syncthreads();
  }
  f = __reduce_or_sync(TC_FULL_MASK, f);
  if ((threadIdx.x & 31) == 0 && f) atomicOr(flags, f);
}

tc_status launch_validate_rowptr(tc_ctx *ctx, const DevCSR &g) {
  validate_rowptr_kernel<<<grid_for(ctx, g.n + 1, 256, 8), 256, 0, ctx->stream>>>(g.rowptr, g.n, g.nnz,
                                                                                  ctx->d_flags);
  TC_CHECK_LAUNCH(ctx);
  return TC_OK;
}

tc_status launch_validate(tc_ctx *ctx, const DevCSR &g, bool simple) {
  TC_TRY(launch_validate_rowptr(ctx, g));
  if (g.nnz > 0) {
    validate_col_kernel<<<grid_for(ctx, g.nnz, ENTRY_TILE, 8), OR_THREADS, 0, ctx->stream>>>(
        g.rowptr, g.col, g.n, g.nnz, simple ? 1 : 0, ctx->d_flags);
    TC_CHECK_LAUNCH(ctx);
  }
  return TC_OK;
}

// ---- phase A: ranks and kept counts ------------------------------------------

__global__ void deg_key_kernel(const int64_t *__restrict__ rowptr, int64_t n, int bits,
                               const int32_t *__restrict__ vgroup, uint64_t *__restrict__ keys) {
  const uint64_t dmax = (bits >= 63) ? ~0ULL : ((1ULL << bits) - 1);
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
    int64_t d = rowptr[u + 1] - rowptr[u];
    uint64_t dd = d < 0 ? 0 : (uint64_t)d;
    if (dd > dmax) dd = dmax;
    const uint64_t grp = vgroup ? (uint64_t)(uint32_t)vgroup[u] : 0;
    keys[u] = (((grp << bits) | dd) << bits) | (uint64_t)u;
  }
}

__global__ void rank_kernel(const uint64_t *__restrict__ keys, int64_t n, uint64_t mask, int32_t *__restrict__ rank) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
    rank[keys[r] & mask] = (int32_t)r;
}

// Kept entries per original row (warp-aggregated atomics) and per block chunk.
// With VALIDATE it also performs validate_col_kernel's checks on the same
// pass over the adjacency (ids in range, rows strictly ascending, no self
// loops), so a validated call reads colidx once here instead of twice.
template <bool VALIDATE>
__global__ void __launch_bounds__(OR_THREADS, 6) kept_count_kernel(const int64_t *__restrict__ rowptr,
                                                               const int32_t *__restrict__ col, int64_t n,
                                                               int64_t nnz, int64_t chunk,
                                                               const int32_t *__restrict__ rank,
                                                               unsigned long long *__restrict__ kept,
                                                               int64_t *__restrict__ bcount, unsigned *flags,
                                                               int b_off, int32_t *__restrict__ rv_out,
                                                               const int32_t *__restrict__ vgroup,
                                                               const int64_t *__restrict__ vtx_off) {
  __shared__ int rows[row_slots<ENTRY_TILE>()];
  __shared__ int scan_tmp[32];
  __shared__ unsigned long long bsum;
  if (threadIdx.x == 0) bsum = 0;
  const int blk = (int)blockIdx.x + b_off;  // block of the entry-chunk geometry
  const int64_t b = (int64_t)blk * chunk, e_end = min(nnz, b + chunk);
  unsigned long long mine = 0;
  unsigned f = 0;
  const int lane = threadIdx.x & 31;
  int64_t hint = -1;
  for (int64_t t0 = b; t0 < e_end; t0 += ENTRY_TILE) {
    const int64_t t1 = min(e_end, t0 + ENTRY_TILE);
    expand_rows<ENTRY_TILE>(rowptr, n, t0, t1, rows, scan_tmp, hint);
    // all loads of the tile first, then the rank gathers, then the counts
    int32_t vv[OR_PER], rv[OR_PER];
#pragma unroll
    for (int k = 0; k < OR_PER; ++k) {
      const int64_t e = t0 + k * OR_THREADS + threadIdx.x;
      vv[k] = e < t1 ? col[e] : -1;
    }
    if (vtx_off) {  // batched graphs: local ids plus the base of the row's graph (always range-checked)
#pragma unroll
      for (int k = 0; k < OR_PER; ++k) {
        const int64_t e = t0 + k * OR_THREADS + threadIdx.x;
        if (e >= t1) continue;
        const int u = rows[rslot((int)(e - t0))];
        int64_t base = 0, size = 0;
        if (u >= 0 && u < n) {
          const int32_t gi = vgroup[u];
          base = vtx_off[gi];
          size = vtx_off[gi + 1] - base;
        }
        if (vv[k] < 0 || (int64_t)vv[k] >= size) {
          f |= VF_ID_RANGE;
          vv[k] = -1;
        } else {
          vv[k] = (int32_t)(base + vv[k]);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < OR_PER; ++k) rv[k] = vv[k] >= 0 && (int64_t)vv[k] < n ? rank[vv[k]] : -1;
    if (rv_out) {  // the placement streams these instead of gathering them again
#pragma unroll
      for (int k = 0; k < OR_PER; ++k) {
        const int64_t e = t0 + k * OR_THREADS + threadIdx.x;
        if (e < t1) rv_out[e] = rv[k];
      }
    }
#pragma unroll
    for (int k = 0; k < OR_PER; ++k) {
      const int64_t e = t0 + k * OR_THREADS + threadIdx.x;
      bool keep = false;
      int u = -1;
      if (e < t1) {
        u = rows[rslot((int)(e - t0))];
        const int32_t v = vv[k];
        keep = u >= 0 && rv[k] >= 0 && rv[k] > rank[u];
        if (VALIDATE) {
          if (v < 0 || (int64_t)v >= n) f |= VF_ID_RANGE;
          else if (u == v) f |= VF_SELF_LOOP;
          // stored ids (local ones in a batch) compare alike within a row
          if (u >= 0 && u < n && e > 0 && e > rowptr[u] && col[e - 1] >= col[e]) f |= VF_UNSORTED;
        }
      }
      // the warp's 32 entries are consecutive, so each row is a run of
      // lanes: the run's first lane adds the run's kept entries
      const unsigned km = __ballot_sync(TC_FULL_MASK, keep);
      const int u_prev = __shfl_up_sync(TC_FULL_MASK, u, 1);
      const bool head = e < t1 && (lane == 0 || u != u_prev);
      const unsigned hm = __ballot_sync(TC_FULL_MASK, head);
      if (head && km) {
        const unsigned later = hm & ~(lanemask_lt() | (1u << lane));  // first lanes of the following runs
        const unsigned run = (later ? (later & (0u - later)) - 1u : 0xffffffffu) & ~lanemask_lt();
        const unsigned c = __popc(km & run);
        if (c) atomicAdd(&kept[u], (unsigned long long)c);
      }
      mine += keep ? 1 : 0;
    }
    __syncthreads();
  }
  mine = warp_sum(mine);
  if (lane == 0 && mine) atomicAdd(&bsum, mine);
  if (VALIDATE || vtx_off) {  // batch ids are range-checked even without validation
    f = __reduce_or_sync(TC_FULL_MASK, f);
    if (lane == 0 && f) atomicOr(flags, f);
  }
  __syncthreads();
  if (threadIdx.x == 0) bcount[blk] = (int64_t)bsum;
}


// Relabelled out-degree (for the row pointers, and with the DAG in-degree,
// the symmetric degree minus the kept out-degree, as one 8-byte pair the
// tile planner gathers per edge target) of every vertex.
__global__ void dnew_kernel(const int64_t *__restrict__ kept, const int32_t *__restrict__ rank,
                            const int64_t *__restrict__ rowptr, int64_t n, int64_t *__restrict__ dnew,
                            int2 *__restrict__ dv) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
    const int32_t r = rank[u];
    const int64_t k = kept[u];
    dnew[r] = k;
    dv[r] = make_int2((int32_t)k, (int32_t)(rowptr[u + 1] - rowptr[u] - k));
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) dnew[n] = 0;
}

// Where the placement puts row u's kept entries: relabelled slot
// rowbase[u] + p for kept entry p (input order) of row u, rowbase[u] =
// nrowptr[rank u] - orowptr[u].  One pass over the vertices, so that the
// placement reads one value per row instead of gathering nrowptr[rank u].
__global__ void rowbase_kernel(const int32_t *__restrict__ rank, const int64_t *__restrict__ nrowptr,
                               const int64_t *__restrict__ orowptr, int64_t n, int64_t *__restrict__ rowbase) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x)
    rowbase[u] = nrowptr[rank[u]] - orowptr[u];
}

// Rows of the relabelled DAG longer than a warp's registers go to list-driven
// sorts: up to SEG_WARP_MAX entries one warp in its own shared-memory slice,
// up to SEG_SMEM_MAX one block in shared memory, beyond that one block in
// place in global memory.  Lists are filled with warp-aggregated atomics
// (their order is irrelevant).
constexpr int SEG_WARP_MAX = 256;
constexpr int SEG_SMEM_MAX = 4096;

__global__ void classify_rows_kernel(const int64_t *__restrict__ len, int64_t n, int32_t *__restrict__ mid_list,
                                     int32_t *__restrict__ big_list, int32_t *__restrict__ huge_list,
                                     unsigned *counts) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = lanemask_lt();
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = base + threadIdx.x;
    const int64_t L = r < n ? len[r] : 0;
#pragma unroll
    for (int cls = 0; cls < 3; ++cls) {
      const bool mine = cls == 0   ? (L > 32 && L <= SEG_WARP_MAX)
                        : cls == 1 ? (L > SEG_WARP_MAX && L <= SEG_SMEM_MAX)
                                   : (L > SEG_SMEM_MAX);
      const unsigned bal = __ballot_sync(TC_FULL_MASK, mine);
      if (!bal) continue;
      unsigned at = 0;
      if (lane == 0) at = atomicAdd(&counts[cls], (unsigned)__popc(bal));
      at = __shfl_sync(TC_FULL_MASK, at, 0);
      int32_t *list = cls == 0 ? mid_list : cls == 1 ? big_list : huge_list;
      if (mine) list[at + __popc(bal & lt)] = (int32_t)r;
    }
  }
}

tc_status orient_phase_a(tc_ctx *ctx, const DevCSR &g, OrientBufs &b) {
  const int bits = vertex_bits(g.n);
  orient_geometry(ctx, g.nnz, b.pieces, &b.G, &b.chunk);
  const int gbits = b.vgroup ? b.group_bits : 0;
  if (2 * bits + gbits > 64) return set_error(ctx, TC_ERR_UNSUPPORTED, "rank key needs %d bits", 2 * bits + gbits);
  deg_key_kernel<<<grid_for(ctx, g.n, 256, 8), 256, 0, ctx->stream>>>(g.rowptr, g.n, bits, b.vgroup, b.vkeys0);
  TC_CHECK_LAUNCH(ctx);
  // Ids start in ascending order and the sort is stable, so sorting on the
  // (group, degree) bits alone yields the (group, degree, id) order.
  uint64_t *sorted = nullptr;
  TC_TRY(radix_sort(ctx, b.vkeys0, b.vkeys1, nullptr, nullptr, g.n, bits, 2 * bits + gbits, b.sort_scratch, &sorted,
                    nullptr));
  rank_kernel<<<grid_for(ctx, g.n, 256, 8), 256, 0, ctx->stream>>>(sorted, g.n, (1ULL << bits) - 1, b.rank);
  TC_CHECK_LAUNCH(ctx);
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(b.kept, 0, sizeof(int64_t) * (size_t)(g.n + 1), ctx->stream));
  if (g.nnz > 0) {
    // one launch per arriving piece of the column array (one piece when it
    // is already on the device); each launch fills the GPU
    const int per = (b.G + b.pieces - 1) / b.pieces;
    for (int k = 0; k < b.pieces && k * per < b.G; ++k) {
      const int blocks = per < b.G - k * per ? per : b.G - k * per;
      if (b.pieces > 1) TC_CHECK_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->piece_ev[k], 0));
      if (b.validate)
        kept_count_kernel<true><<<blocks, OR_THREADS, 0, ctx->stream>>>(g.rowptr, g.col, g.n, g.nnz, b.chunk,
                                                                        b.rank, (unsigned long long *)b.kept,
                                                                        b.bcount, ctx->d_flags, k * per, b.rv,
                                                                        b.vgroup, b.vtx_off);
      else
        kept_count_kernel<false><<<blocks, OR_THREADS, 0, ctx->stream>>>(g.rowptr, g.col, g.n, g.nnz, b.chunk,
                                                                         b.rank, (unsigned long long *)b.kept,
                                                                         b.bcount, ctx->d_flags, k * per, b.rv,
                                                                         b.vgroup, b.vtx_off);
      TC_CHECK_LAUNCH(ctx);
    }
    TC_TRY(exclusive_scan_i64(ctx, b.bcount, b.bcount, b.G, b.sort_scratch, b.d_m));
  } else {
    TC_CHECK_CUDA(ctx, cudaMemsetAsync(b.d_m, 0, sizeof(int64_t), ctx->stream));
  }
  // original-order DAG rowptr, relabelled rowptr, and the row classes
  TC_TRY(exclusive_scan_i64(ctx, b.kept, b.orowptr, g.n + 1, b.sort_scratch, nullptr));
  dnew_kernel<<<grid_for(ctx, g.n, 256, 8), 256, 0, ctx->stream>>>(b.kept, b.rank, g.rowptr, g.n, b.dnew,
                                                                    b.dv);
  TC_CHECK_LAUNCH(ctx);
  TC_TRY(exclusive_scan_i64(ctx, b.dnew, b.nrowptr, g.n + 1, b.sort_scratch, nullptr));
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(b.seg_counts, 0, sizeof(unsigned) * 4, ctx->stream));
  classify_rows_kernel<<<grid_for(ctx, g.n, 256, 8), 256, 0, ctx->stream>>>(b.dnew, g.n, b.mid_list, b.big_list,
                                                                            b.huge_list, b.seg_counts);
  TC_CHECK_LAUNCH(ctx);
  if (PLACE_ROWBASE) {  // into b.kept, whose counts are spent once orowptr and dnew are made
    rowbase_kernel<<<grid_for(ctx, g.n, 256, 8), 256, 0, ctx->stream>>>(b.rank, b.nrowptr, b.orowptr, g.n, b.kept);
    TC_CHECK_LAUNCH(ctx);
  }
  return TC_OK;
}

// ---- phase B: direct placement + per-row sort ---------------------------------

// Kept entry k (input order, original slot kpos) of row u goes to relabelled
// slot nrowptr[rank u] + (kpos - orowptr[u]) with value rank v; rows are then
// sorted by value.
template <bool VALS, bool DAGCOL, bool RELABEL>
__global__ void __launch_bounds__(OR_THREADS, 6) place_kernel(const int64_t *__restrict__ rowptr,
                                                          const int32_t *__restrict__ col, int64_t n, int64_t nnz,
                                                          int64_t chunk, const int32_t *__restrict__ rank,
                                                          const int64_t *__restrict__ boff,
                                                          const int64_t *__restrict__ orowptr,
                                                          const int64_t *__restrict__ nrowptr,
                                                          int32_t *__restrict__ ncol, int32_t *__restrict__ nsrc,
                                                          uint32_t *__restrict__ perm,
                                                          int32_t *__restrict__ dag_col,
                                                          const int32_t *__restrict__ rv_in,
                                                          const int64_t *__restrict__ rowbase) {
  __shared__ int rows[row_slots<ENTRY_TILE>()];
  __shared__ int scan_tmp[32];
  __shared__ long long s_wbase[OR_THREADS / 32 + 1];
  constexpr int NW = OR_THREADS / 32;
  const int64_t b = (int64_t)blockIdx.x * chunk, e_end = min(nnz, b + chunk);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = lanemask_lt();
  long long carry = boff[blockIdx.x];
  int64_t hint = -1;
  for (int64_t t0 = b; t0 < e_end; t0 += ENTRY_TILE) {
    const int64_t t1 = min(e_end, t0 + ENTRY_TILE);
    expand_rows<ENTRY_TILE>(rowptr, n, t0, t1, rows, scan_tmp, hint);
    // warp w owns entries [w*32*OR_PER, (w+1)*32*OR_PER) of the tile, lane-
    // strided so every load is coalesced; entry order = (k, lane) order
    const int wbase = warp * 32 * OR_PER;
    int32_t vv[OR_PER], rv[OR_PER], uu[OR_PER];
#pragma unroll
    for (int k = 0; k < OR_PER; ++k) {
      const int i = wbase + k * 32 + lane;
      const bool in = t0 + i < t1;
      vv[k] = in && (DAGCOL || !rv_in) ? col[t0 + i] : -1;
      uu[k] = in ? rows[rslot(i)] : -1;
      if (rv_in) rv[k] = in ? rv_in[t0 + i] : -1;  // ranks of the targets, from the kept-count pass
    }
    if (!rv_in) {
#pragma unroll
      for (int k = 0; k < OR_PER; ++k) rv[k] = vv[k] >= 0 && (int64_t)vv[k] < n ? rank[vv[k]] : -1;
    }
    unsigned bal[OR_PER];
    int cnt = 0;
#pragma unroll
    for (int k = 0; k < OR_PER; ++k) {
      const bool keep = uu[k] >= 0 && rv[k] >= 0 && rv[k] > rank[uu[k]];
      bal[k] = __ballot_sync(TC_FULL_MASK, keep);
      cnt += __popc(bal[k]);
    }
    if (lane == 0) s_wbase[warp] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
      long long acc = 0;
      for (int w = 0; w < NW; ++w) {
        const long long c = s_wbase[w];
        s_wbase[w] = acc;
        acc += c;
      }
      s_wbase[NW] = acc;
    }
    __syncthreads();
    long long pos = carry + s_wbase[warp];
#pragma unroll
    for (int k = 0; k < OR_PER; ++k) {
      if ((bal[k] >> lane) & 1u) {
        const long long p = pos + __popc(bal[k] & lt);
        const int u = uu[k];
        if (RELABEL) {
          const long long dst = PLACE_ROWBASE ? rowbase[u] + p : nrowptr[rank[u]] + (p - orowptr[u]);
          ncol[dst] = rv[k];
          if (PLACE_SRC) nsrc[dst] = rank[u];
          if (VALS) perm[dst] = (uint32_t)p;
        }
        if (DAGCOL) dag_col[p] = vv[k];
      }
      pos += __popc(bal[k]);
    }
    carry += s_wbase[NW];
    __syncthreads();
  }
}

// Ascending bitonic network in its "flip" form: every comparator puts the
// smaller key at the lower index, so a list of any length L behaves as if
// padded with +infinity and comparators reaching past L are skipped.
template <bool VALS>
__device__ __forceinline__ void cmp_swap(int32_t *key, uint32_t *val, int a, int b) {
  const int32_t ka = key[a], kb = key[b];
  if (kb < ka) {
    key[a] = kb;
    key[b] = ka;
    if (VALS) {
      const uint32_t t = val[a];
      val[a] = val[b];
      val[b] = t;
    }
  }
}

template <bool VALS>
__device__ void block_flip_bitonic(int32_t *key, uint32_t *val, int L) {
  int P = 1;
  while (P < L) P <<= 1;
  for (int k = 2; k <= P; k <<= 1) {
    const int h = k >> 1;
    for (int t = threadIdx.x; t < P / 2; t += blockDim.x) {
      const int blk = t / h, off = t % h;
      const int a = blk * k + off, bb = blk * k + k - 1 - off;
      if (bb < L) cmp_swap<VALS>(key, val, a, bb);
    }
    __syncthreads();
    for (int j = k >> 2; j >= 1; j >>= 1) {
      for (int t = threadIdx.x; t < P / 2; t += blockDim.x) {
        const int a = (t / j) * 2 * j + (t % j), bb = a + j;
        if (bb < L) cmp_swap<VALS>(key, val, a, bb);
      }
      __syncthreads();
    }
  }
}

// Register stages of the same network for one 32-entry chunk (one warp):
// chunk_sort32 runs levels 2..32 completely; chunk_merge32 runs the
// comparators at distances 16..1 of a later level (all ascending).  Slots at
// or beyond L read as +infinity and are not written back.
template <bool VALS>
__device__ __forceinline__ void reg_cmp(int32_t &key, uint32_t &val, int lane, int partner) {
  const int32_t ok = __shfl_sync(TC_FULL_MASK, key, partner);
  const uint32_t ov = VALS ? __shfl_sync(TC_FULL_MASK, val, partner) : 0u;
  const bool take = lane < partner ? ok < key : ok > key;
  if (take) {
    key = ok;
    if (VALS) val = ov;
  }
}

template <bool VALS, bool FULL>
__device__ __forceinline__ void chunk_stages32(int32_t *key, uint32_t *val, int c0, int L, int lane) {
  const int i = c0 + lane;
  int32_t k = i < L ? key[i] : INT32_MAX;
  uint32_t v = (VALS && i < L) ? val[i] : 0u;
  if (FULL) {
#pragma unroll
    for (int lv = 2; lv <= 32; lv <<= 1) {
      reg_cmp<VALS>(k, v, lane, lane ^ (lv - 1));
#pragma unroll
      for (int j = lv >> 2; j >= 1; j >>= 1) reg_cmp<VALS>(k, v, lane, lane ^ j);
    }
  } else {
#pragma unroll
    for (int j = 16; j >= 1; j >>= 1) reg_cmp<VALS>(k, v, lane, lane ^ j);
  }
  if (i < L) {
    key[i] = k;
    if (VALS) val[i] = v;
  }
}

// The flip network for a list in shared memory of up to 32 * 32 * blocks
// entries, by the block (SYNC_BLOCK) or by one warp: stages with comparator
// distance >= 32 in shared memory, the rest in registers, 32 entries per
// warp at a time.
template <bool VALS, bool SYNC_BLOCK>
__device__ void hybrid_flip_bitonic(int32_t *key, uint32_t *val, int L, int warp, int nwarps, int lane) {
  int P = 32;
  while (P < L) P <<= 1;
  const int nth = SYNC_BLOCK ? (int)blockDim.x : 32, tid = SYNC_BLOCK ? (int)threadIdx.x : lane;
  for (int c0 = warp * 32; c0 < P; c0 += nwarps * 32) chunk_stages32<VALS, true>(key, val, c0, L, lane);
  if (SYNC_BLOCK) __syncthreads(); else __syncwarp();
  for (int k = 64; k <= P; k <<= 1) {
    const int h = k >> 1;
    for (int t = tid; t < P / 2; t += nth) {
      const int blk = t / h, off = t % h;
      const int a = blk * k + off, bb = blk * k + k - 1 - off;
      if (bb < L) cmp_swap<VALS>(key, val, a, bb);
    }
    if (SYNC_BLOCK) __syncthreads(); else __syncwarp();
    for (int j = k >> 2; j >= 32; j >>= 1) {
      for (int t = tid; t < P / 2; t += nth) {
        const int a = (t / j) * 2 * j + (t % j), bb = a + j;
        if (bb < L) cmp_swap<VALS>(key, val, a, bb);
      }
      if (SYNC_BLOCK) __syncthreads(); else __syncwarp();
    }
    for (int c0 = warp * 32; c0 < P; c0 += nwarps * 32) chunk_stages32<VALS, false>(key, val, c0, L, lane);
    if (SYNC_BLOCK) __syncthreads(); else __syncwarp();
  }
}

template <bool VALS>
__global__ void seg_sort_warp_kernel(const int64_t *__restrict__ nrowptr, int64_t n, int32_t *__restrict__ ncol,
                                     uint32_t *__restrict__ perm, int32_t *__restrict__ src) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
    const int64_t b = nrowptr[r];
    const int L = (int)(nrowptr[r + 1] - b);
    if (L <= 32) put_row_src(src, b, L, (int32_t)r, lane, 32);
    if (L < 2 || L > 32) continue;
    int32_t key = lane < L ? ncol[b + lane] : INT32_MAX;
    uint32_t val = (VALS && lane < L) ? perm[b + lane] : 0u;
    int P = 2;  // levels up to the row's padded length only (warp-uniform)
    while (P < L) P <<= 1;
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
      if (k > P) break;
      {
        const int partner = lane ^ (k - 1);
        const int32_t ok = __shfl_sync(TC_FULL_MASK, key, partner);
        const uint32_t ov = VALS ? __shfl_sync(TC_FULL_MASK, val, partner) : 0u;
        const bool take = lane < partner ? ok < key : ok > key;
        if (take) { key = ok; if (VALS) val = ov; }
      }
#pragma unroll
      for (int j = k >> 2; j >= 1; j >>= 1) {
        const int partner = lane ^ j;
        const int32_t ok = __shfl_sync(TC_FULL_MASK, key, partner);
        const uint32_t ov = VALS ? __shfl_sync(TC_FULL_MASK, val, partner) : 0u;
        const bool take = lane < partner ? ok < key : ok > key;
        if (take) { key = ok; if (VALS) val = ov; }
      }
    }
    if (lane < L) {
      ncol[b + lane] = key;
      if (VALS) perm[b + lane] = val;
    }
  }
}

// The same sort with a warp per 32 consecutive rows: the warp reads their 33
// row pointers with one coalesced load, then sorts the rows one after
// another, loading the next row while it sorts the current one, so a row
// costs one memory round trip instead of the two dependent ones (its
// pointers, then its entries) of a warp per row.
template <bool VALS>
__device__ __forceinline__ void warp_sort32(int32_t &key, uint32_t &val, int L, int lane) {
  int P = 2;  // levels up to the row's padded length only (warp-uniform)
  while (P < L) P <<= 1;
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
    if (k > P) break;
    {
      const int partner = lane ^ (k - 1);
      const int32_t ok = __shfl_sync(TC_FULL_MASK, key, partner);
      const uint32_t ov = VALS ? __shfl_sync(TC_FULL_MASK, val, partner) : 0u;
      const bool take = lane < partner ? ok < key : ok > key;
      if (take) { key = ok; if (VALS) val = ov; }
    }
#pragma unroll
    for (int j = k >> 2; j >= 1; j >>= 1) {
      const int partner = lane ^ j;
      const int32_t ok = __shfl_sync(TC_FULL_MASK, key, partner);
      const uint32_t ov = VALS ? __shfl_sync(TC_FULL_MASK, val, partner) : 0u;
      const bool take = lane < partner ? ok < key : ok > key;
      if (take) { key = ok; if (VALS) val = ov; }
    }
  }
}

template <bool VALS>
__global__ void seg_sort_warp_chunk_kernel(const int64_t *__restrict__ nrowptr, int64_t n,
                                           int32_t *__restrict__ ncol, uint32_t *__restrict__ perm,
                                           int32_t *__restrict__ src) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; r0 < n; r0 += warps * 32) {
    const int64_t rl = min(r0 + lane, n);  // lane's row start (row n: the end)
    const int64_t lo_l = nrowptr[rl];
    const int64_t hi_l = nrowptr[min(rl + 1, n)];
    const int rows = (int)min((int64_t)32, n - r0);
    // prefetch the first row
    int64_t b = __shfl_sync(TC_FULL_MASK, lo_l, 0);
    int L = (int)(__shfl_sync(TC_FULL_MASK, hi_l, 0) - b);
    int32_t key = (L >= 2 && L <= 32 && lane < L) ? ncol[b + lane] : INT32_MAX;
    uint32_t val = (VALS && L >= 2 && L <= 32 && lane < L) ? perm[b + lane] : 0u;
    for (int j = 0; j < rows; ++j) {
      const int64_t bj = b;
      const int Lj = L;
      int32_t kj = key;
      uint32_t vj = val;
      if (j + 1 < rows) {  // next row's entries in flight while this one sorts
        b = __shfl_sync(TC_FULL_MASK, lo_l, j + 1);
        L = (int)(__shfl_sync(TC_FULL_MASK, hi_l, j + 1) - b);
        key = (L >= 2 && L <= 32 && lane < L) ? ncol[b + lane] : INT32_MAX;
        val = (VALS && L >= 2 && L <= 32 && lane < L) ? perm[b + lane] : 0u;
      }
      if (Lj <= 32) put_row_src(src, bj, Lj, (int32_t)(r0 + j), lane, 32);
      if (Lj < 2 || Lj > 32) continue;  // warp-uniform
      warp_sort32<VALS>(kj, vj, Lj, lane);
      if (lane < Lj) {
        ncol[bj + lane] = kj;
        if (VALS) perm[bj + lane] = vj;
      }
    }
  }
}

// The flip network over 32 * E keys held E per lane in registers, lane l
// holding entries [l*E, l*E + E): comparators between entries of one lane
// are register compare-exchanges; between lanes, each lane trades one key
// per entry with one shuffle and keeps the smaller (lower entry) or larger.
// Entry i's flip partner at level lv is i ^ (lv - 1), i.e. lane l ^ (lv/E -
// 1), slot E - 1 - x; its half-cleaner partner at distance j is i ^ j.
template <bool VALS>
__device__ __forceinline__ void reg_keep(int32_t &k, uint32_t &v, int32_t ok, uint32_t ov, bool lower) {
  if (lower ? ok < k : ok > k) {
    k = ok;
    if (VALS) v = ov;
  }
}

template <int E, bool VALS>
__device__ __forceinline__ void warp_sort_blocked(int32_t (&k)[E], uint32_t (&v)[E], int lane) {
  static_assert(E >= 2 && (E & (E - 1)) == 0, "2, 4, 8, ... keys per lane");
  constexpr int P = 32 * E;
#pragma unroll
  for (int lv = 2; lv <= P; lv <<= 1) {
    if (lv <= E) {
#pragma unroll
      for (int x = 0; x < E; ++x) {
        const int y = x ^ (lv - 1);
        if (y > x && k[y] < k[x]) {
          const int32_t t = k[x];
          k[x] = k[y];
          k[y] = t;
          if (VALS) {
            const uint32_t s = v[x];
            v[x] = v[y];
            v[y] = s;
          }
        }
      }
    } else {
      // entries x and E-1-x trade with the partner's E-1-x and x: both keys
      // are read before either is replaced, so no second key array is held
      const int pl = lane ^ (lv / E - 1);
      const bool lower = ((lane * E) & (lv >> 1)) == 0;
#pragma unroll
      for (int x = 0; x < E / 2; ++x) {
        const int y = E - 1 - x;
        const int32_t o1 = __shfl_sync(TC_FULL_MASK, k[y], pl), o2 = __shfl_sync(TC_FULL_MASK, k[x], pl);
        const uint32_t w1 = VALS ? __shfl_sync(TC_FULL_MASK, v[y], pl) : 0u;
        const uint32_t w2 = VALS ? __shfl_sync(TC_FULL_MASK, v[x], pl) : 0u;
        reg_keep<VALS>(k[x], v[x], o1, w1, lower);
        reg_keep<VALS>(k[y], v[y], o2, w2, lower);
      }
    }
#pragma unroll
    for (int j = lv >> 2; j >= 1; j >>= 1) {
      if (j < E) {
#pragma unroll
        for (int x = 0; x < E; ++x) {
          if (x & j) continue;
          const int y = x | j;
          if (k[y] < k[x]) {
            const int32_t t = k[x];
            k[x] = k[y];
            k[y] = t;
            if (VALS) {
              const uint32_t s = v[x];
              v[x] = v[y];
              v[y] = s;
            }
          }
        }
      } else {
        const int pl = lane ^ (j / E);
        const bool lower = ((lane * E) & j) == 0;
#pragma unroll
        for (int x = 0; x < E; ++x) {
          const int32_t o = __shfl_sync(TC_FULL_MASK, k[x], pl);
          const uint32_t w = VALS ? __shfl_sync(TC_FULL_MASK, v[x], pl) : 0u;
          reg_keep<VALS>(k[x], v[x], o, w, lower);
        }
      }
    }
  }
}

template <int E, bool VALS>
__device__ __forceinline__ void warp_sort_row_blocked(int32_t *__restrict__ ncol, uint32_t *__restrict__ perm,
                                                      int64_t b, int L, int lane) {
  int32_t k[E];
  uint32_t v[E];
#pragma unroll
  for (int x = 0; x < E; ++x) {
    const int i = lane * E + x;
    k[x] = i < L ? ncol[b + i] : INT32_MAX;
    v[x] = (VALS && i < L) ? perm[b + i] : 0u;
  }
  warp_sort_blocked<E, VALS>(k, v, lane);
#pragma unroll
  for (int x = 0; x < E; ++x) {
    const int i = lane * E + x;
    if (i < L) {
      ncol[b + i] = k[x];
      if (VALS) perm[b + i] = v[x];
    }
  }
}

// Rows of 33..SEG_WARP_MAX entries: one warp per row, 2, 4 or 8 keys per
// lane in registers (warp_sort_blocked).
template <bool VALS>
__global__ void __launch_bounds__(256) seg_sort_warpreg_kernel(const int64_t *__restrict__ nrowptr,
                                                              const int32_t *__restrict__ list,
                                                              const unsigned *count, int32_t *__restrict__ ncol,
                                                              uint32_t *__restrict__ perm, int32_t *__restrict__ src) {
  static_assert(SEG_WARP_MAX == 256, "rows of up to 8 keys per lane");
  const int lane = threadIdx.x & 31;
  const unsigned cnt = *count;
  const unsigned warps = gridDim.x * (blockDim.x >> 5);
  for (unsigned i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < cnt; i += warps) {
    const int32_t r = list[i];
    const int64_t b = nrowptr[r];
    const int L = (int)(nrowptr[r + 1] - b);
    if (L <= 64) warp_sort_row_blocked<2, VALS>(ncol, perm, b, L, lane);
    else if (L <= 128) warp_sort_row_blocked<4, VALS>(ncol, perm, b, L, lane);
    else warp_sort_row_blocked<8, VALS>(ncol, perm, b, L, lane);
    put_row_src(src, b, L, r, lane, 32);
  }
}

// Rows of SEG_WARP_MAX+1..SEG_SMEM_MAX entries without payload whose ids
// span at most WB_WORDS * 32 values: one warp per row sorts through a
// bitmap in its own 4 KB of shared memory, with no block barrier (most such
// rows have a few hundred entries, too few to keep a block busy between its
// barriers).  Bits are set with atomicOr; a total popcount different from
// the row's length means duplicate ids (unvalidated input only).  Then the
// words are read back 32 at a time, one per lane, and a warp prefix sum of
// their popcounts gives each lane where its word's ids go, in order; each
// word is zeroed as it is read.  Rows that do not fit (wider windows,
// duplicates) are appended to `defer` for seg_sort_smem_kernel.
constexpr int WB_WORDS = 1024;
constexpr int WB_WARPS = 8;

__global__ void __launch_bounds__(WB_WARPS * 32) seg_sort_warpbits_kernel(const int64_t *__restrict__ nrowptr,
                                                                         const int32_t *__restrict__ list,
                                                                         const unsigned *count,
                                                                         int32_t *__restrict__ ncol,
                                                                         int32_t *__restrict__ defer,
                                                                         unsigned *defer_count,
                                                                         int32_t *__restrict__ src) {
  __shared__ uint32_t bits_all[WB_WARPS][WB_WORDS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t *bm = bits_all[w];
  for (int q = lane; q < WB_WORDS; q += 32) bm[q] = 0u;
  __syncwarp();
  const unsigned cnt = *count;
  const unsigned warps = gridDim.x * WB_WARPS;
  for (unsigned i = blockIdx.x * WB_WARPS + w; i < cnt; i += warps) {
    const int32_t r = list[i];
    const int64_t b = nrowptr[r];
    const int L = (int)(nrowptr[r + 1] - b);
    int32_t lo = INT32_MAX, hi = INT32_MIN;
    for (int k = lane; k < L; k += 32) {
      const int32_t x = ncol[b + k];
      lo = min(lo, x);
      hi = max(hi, x);
    }
    lo = __reduce_min_sync(TC_FULL_MASK, lo);
    hi = __reduce_max_sync(TC_FULL_MASK, hi);
    const int64_t span = (int64_t)hi - lo + 1;
    bool fits = L > 0 && span <= (int64_t)WB_WORDS * 32;
    const int W = fits ? (int)((span + 31) >> 5) : 0;
    if (fits) {
      for (int k = lane; k < L; k += 32) {
        const uint32_t d = (uint32_t)(ncol[b + k] - lo);
        atomicOr(&bm[d >> 5], 1u << (d & 31));
      }
      __syncwarp();
      int c = 0;
      for (int q = lane; q < W; q += 32) c += __popc(bm[q]);
      fits = __reduce_add_sync(TC_FULL_MASK, (unsigned)c) == (unsigned)L;
      if (!fits) {  // duplicate ids: clear, then leave the row to the block sort
        __syncwarp();
        for (int q = lane; q < W; q += 32) bm[q] = 0u;
      }
    }
    if (!fits) {  // wider window (or duplicate ids): left to the block sort
      if (lane == 0) defer[atomicAdd(defer_count, 1u)] = r;
      __syncwarp();
      continue;
    }
    int base = 0;
    for (int q0 = 0; q0 < W; q0 += 32) {
      const int q = q0 + lane;
      uint32_t word = q < W ? bm[q] : 0u;
      if (q < W) bm[q] = 0u;
      const int pc = __popc(word);
      int incl = pc;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(TC_FULL_MASK, incl, o);
        if (lane >= o) incl += t;
      }
      int at = base + incl - pc;
      while (word) {
        const int bit = __ffs(word) - 1;
        word &= word - 1u;
        ncol[b + at++] = lo + 32 * q + bit;
      }
      base += __shfl_sync(TC_FULL_MASK, incl, 31);
    }
    put_row_src(src, b, L, r, lane, 32);
    __syncwarp();
  }
}

// Rows of 33..SEG_WARP_MAX entries: one warp per row sorts in its own slice
// of shared memory with the same flip network (register stages for
// distances below 32), synchronising with __syncwarp.
template <bool VALS>
__global__ void __launch_bounds__(256) seg_sort_warpsmem_kernel(const int64_t *__restrict__ nrowptr,
                                                               const int32_t *__restrict__ list,
                                                               const unsigned *count, int32_t *__restrict__ ncol,
                                                               uint32_t *__restrict__ perm, int32_t *__restrict__ src) {
  __shared__ int32_t skey_all[8][SEG_WARP_MAX];
  __shared__ uint32_t sval_all[VALS ? 8 : 1][VALS ? SEG_WARP_MAX : 1];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t *key = skey_all[w];
  uint32_t *val = VALS ? sval_all[w] : nullptr;
  const unsigned cnt = *count;
  const unsigned warps = gridDim.x * (blockDim.x >> 5);
  for (unsigned i = blockIdx.x * (blockDim.x >> 5) + w; i < cnt; i += warps) {
    const int32_t r = list[i];
    const int64_t b = nrowptr[r];
    const int L = (int)(nrowptr[r + 1] - b);
    for (int k = lane; k < L; k += 32) {
      key[k] = ncol[b + k];
      if (VALS) val[k] = perm[b + k];
    }
    __syncwarp();
    hybrid_flip_bitonic<VALS, false>(key, val, L, 0, 1, lane);
    for (int k = lane; k < L; k += 32) {
      ncol[b + k] = key[k];
      if (VALS) perm[b + k] = val[k];
    }
    put_row_src(src, b, L, r, lane, 32);
    __syncwarp();
  }
}

// Rows without payload whose ids span at most SEG_SMEM_MAX * 32 values are
// sorted through a bitmap in the key buffer: one bit per entry (a row's ids
// are distinct), a block prefix of the words' popcounts, then every thread
// writes its words' set bits in order.
constexpr int SEG_BITMAP_KEYS = SEG_SMEM_MAX / 256;  // keys per thread (256 threads)

template <bool VALS>
__global__ void __launch_bounds__(256) seg_sort_smem_kernel(const int64_t *__restrict__ nrowptr,
                                                           const int32_t *__restrict__ list, const unsigned *count,
                                                           int32_t *__restrict__ ncol, uint32_t *__restrict__ perm,
                                                           int32_t *__restrict__ src) {
  __shared__ int32_t skey[SEG_SMEM_MAX];
  __shared__ uint32_t sval[VALS ? SEG_SMEM_MAX : 1];
  __shared__ int32_t s_red[2][8];
  __shared__ int32_t s_wsum[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned cnt = *count;
  for (unsigned i = blockIdx.x; i < cnt; i += gridDim.x) {
    const int32_t r = list[i];
    const int64_t b = nrowptr[r];
    const int L = (int)(nrowptr[r + 1] - b);
    put_row_src(src, b, L, r, threadIdx.x, blockDim.x);  // the row's entries stay in it
    if (!VALS) {
      int32_t x[SEG_BITMAP_KEYS];
      int32_t lo = 0x7fffffff, hi = -1;
#pragma unroll
      for (int j = 0; j < SEG_BITMAP_KEYS; ++j) {
        const int k = (int)threadIdx.x + 256 * j;
        x[j] = k < L ? ncol[b + k] : -1;
        if (k < L) {
          lo = min(lo, x[j]);
          hi = max(hi, x[j]);
        }
      }
      lo = __reduce_min_sync(TC_FULL_MASK, lo);
      hi = __reduce_max_sync(TC_FULL_MASK, hi);
      if (lane == 0) {
        s_red[0][warp] = lo;
        s_red[1][warp] = hi;
      }
      __syncthreads();
      lo = s_red[0][0];
      hi = s_red[1][0];
#pragma unroll
      for (int w = 1; w < 8; ++w) {
        lo = min(lo, s_red[0][w]);
        hi = max(hi, s_red[1][w]);
      }
      const int64_t span = (int64_t)hi - lo + 1;
      if (span <= (int64_t)SEG_SMEM_MAX * 32) {  // uniform over the block
        const int W = (int)((span + 31) >> 5);
        uint32_t *bm = reinterpret_cast<uint32_t *>(skey);
        for (int q = threadIdx.x; q < W; q += 256) bm[q] = 0u;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < SEG_BITMAP_KEYS; ++j)
          if ((int)threadIdx.x + 256 * j < L) {
            const int d = x[j] - lo;
            atomicOr(&bm[d >> 5], 1u << (d & 31));
          }
        __syncthreads();
        // thread t owns words [t * per, (t + 1) * per)
        const int per = (W + 255) / 256;
        const int w0 = min(W, (int)threadIdx.x * per), w1 = min(W, w0 + per);
        int c = 0;
        for (int q = w0; q < w1; ++q) c += __popc(bm[q]);
        int inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(TC_FULL_MASK, inc, o);
          if (lane >= o) inc += y;
        }
        if (lane == 31) s_wsum[warp] = inc;
        __syncthreads();
        int pos = inc - c, total = 0;
        for (int w = 0; w < 8; ++w) {
          if (w < warp) pos += s_wsum[w];
          total += s_wsum[w];
        }
        if (total != L) {  // duplicate ids (only without validation): keep them, sort by comparisons
          __syncthreads();
#pragma unroll
          for (int j = 0; j < SEG_BITMAP_KEYS; ++j)
            if ((int)threadIdx.x + 256 * j < L) skey[threadIdx.x + 256 * j] = x[j];
          __syncthreads();
          hybrid_flip_bitonic<VALS, true>(skey, sval, L, warp, blockDim.x >> 5, lane);
          for (int k = threadIdx.x; k < L; k += blockDim.x) ncol[b + k] = skey[k];
          __syncthreads();
          continue;
        }
        for (int q = w0; q < w1; ++q) {
          uint32_t bits = bm[q];
          while (bits) {
            const int t = __ffs(bits) - 1;
            bits &= bits - 1;
            ncol[b + pos++] = lo + 32 * q + t;
          }
        }
        __syncthreads();
        continue;
      }
      __syncthreads();  // s_red is read again by the next row
    }
    for (int k = threadIdx.x; k < L; k += blockDim.x) {
      skey[k] = ncol[b + k];
      if (VALS) sval[k] = perm[b + k];
    }
    __syncthreads();
    hybrid_flip_bitonic<VALS, true>(skey, sval, L, threadIdx.x >> 5, blockDim.x >> 5, threadIdx.x & 31);
    for (int k = threadIdx.x; k < L; k += blockDim.x) {
      ncol[b + k] = skey[k];
      if (VALS) perm[b + k] = sval[k];
    }
    __syncthreads();
  }
}

template <bool VALS>
__global__ void __launch_bounds__(1024) seg_sort_global_kernel(const int64_t *__restrict__ nrowptr,
                                                              const int32_t *__restrict__ list, const unsigned *count,
                                                              int32_t *ncol, uint32_t *perm, int32_t *src) {
  const unsigned cnt = *count;
  for (unsigned i = blockIdx.x; i < cnt; i += gridDim.x) {
    const int32_t r = list[i];
    const int64_t b = nrowptr[r];
    const int L = (int)(nrowptr[r + 1] - b);
    put_row_src(src, b, L, r, threadIdx.x, blockDim.x);
    block_flip_bitonic<VALS>(ncol + b, VALS ? perm + b : nullptr, L);
    __syncthreads();
  }
}

// Sorts every relabelled row by target rank: rows of <= 32 entries in
// registers, then the three list-driven classes.
template <bool VALS>
static tc_status launch_row_sorts(tc_ctx *ctx, const DevCSR &g, OrientBufs &b) {
  uint32_t *pv = VALS ? b.perm : nullptr;
  int32_t *sv = SORT_SRC ? b.nsrc : nullptr;  // rows written by the sorts (every row visits one)
  if (SEG_WARP_CHUNK)
    seg_sort_warp_chunk_kernel<VALS><<<grid_for(ctx, g.n, 256, 8), 256, 0, ctx->stream>>>(b.nrowptr, g.n, b.ncol,
                                                                                          pv, sv);
  else
    seg_sort_warp_kernel<VALS><<<grid_for(ctx, g.n * 32, 256, 8), 256, 0, ctx->stream>>>(b.nrowptr, g.n, b.ncol, pv,
                                                                                         sv);
  TC_CHECK_LAUNCH(ctx);
  if (SEG_WARP_REG)
    seg_sort_warpreg_kernel<VALS><<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(b.nrowptr, b.mid_list, b.seg_counts,
                                                                            b.ncol, pv, sv);
  else
    seg_sort_warpsmem_kernel<VALS><<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(b.nrowptr, b.mid_list, b.seg_counts,
                                                                            b.ncol, pv, sv);
  TC_CHECK_LAUNCH(ctx);
  if (!VALS && SEG_WARP_BITS) {
    // narrow rows through warp bitmaps; the rest (deferred into mid_list,
    // which the warp sort above has finished with) through the block sort
    seg_sort_warpbits_kernel<<<ctx->num_sms * 4, WB_WARPS * 32, 0, ctx->stream>>>(
        b.nrowptr, b.big_list, b.seg_counts + 1, b.ncol, b.mid_list, b.seg_counts + 3, sv);
    TC_CHECK_LAUNCH(ctx);
    seg_sort_smem_kernel<VALS><<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(b.nrowptr, b.mid_list, b.seg_counts + 3,
                                                                          b.ncol, pv, sv);
  } else {
    seg_sort_smem_kernel<VALS><<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(b.nrowptr, b.big_list, b.seg_counts + 1,
                                                                          b.ncol, pv, sv);
  }
  TC_CHECK_LAUNCH(ctx);
  seg_sort_global_kernel<VALS><<<ctx->num_sms, 1024, 0, ctx->stream>>>(b.nrowptr, b.huge_list, b.seg_counts + 2,
                                                                       b.ncol, pv, sv);
  TC_CHECK_LAUNCH(ctx);
  return TC_OK;
}

tc_status orient_phase_b(tc_ctx *ctx, const DevCSR &g, OrientBufs &b, int64_t m, bool want_perm, bool want_dag_cols,
                         DevDag *out) {
  const bool relabel = out != nullptr;
  if (g.nnz > 0 && m > 0) {
#define TC_PLACE(V, D, R)                                                                                        \
  place_kernel<V, D, R><<<b.G, OR_THREADS, 0, ctx->stream>>>(g.rowptr, g.col, g.n, g.nnz, b.chunk, b.rank, b.bcount, \
                                                             b.orowptr, b.nrowptr, b.ncol, b.nsrc, b.perm, b.dag_col, \
                                                             b.rv, b.kept)
    if (!relabel) TC_PLACE(false, true, false);
    else if (want_perm && want_dag_cols) TC_PLACE(true, true, true);
    else if (want_perm) TC_PLACE(true, false, true);
    else if (want_dag_cols) TC_PLACE(false, true, true);
    else TC_PLACE(false, false, true);
#undef TC_PLACE
    TC_CHECK_LAUNCH(ctx);
  }
  if (!relabel) return TC_OK;
  // the row sorts keep entries inside their rows, so every entry's row
  // (nsrc) is the same before and after them
  if (m > 1) TC_TRY(want_perm ? launch_row_sorts<true>(ctx, g, b) : launch_row_sorts<false>(ctx, g, b));
  if (TC_PLACE_SRC == 0 || (SORT_SRC && m <= 1)) TC_TRY(launch_expand_src(ctx, b.nrowptr, g.n, m, b.nsrc));
  out->n = g.n;
  out->m = m;
  out->rowptr = b.nrowptr;
  out->col = b.ncol;
  out->src = b.nsrc;
  out->perm = want_perm ? b.perm : nullptr;
  out->indeg = nullptr;
  out->dv = b.dv;
  out->restrict_after = 1;
  return TC_OK;
}

// ---- row of each entry (for caller-oriented DAGs) -----------------------------

__global__ void __launch_bounds__(OR_THREADS) expand_src_kernel(const int64_t *__restrict__ rowptr, int64_t n,
                                                               int64_t m, int32_t *__restrict__ src) {
  __shared__ int rows[row_slots<ENTRY_TILE>()];
  __shared__ int scan_tmp[32];
  const int64_t tiles = (m + ENTRY_TILE - 1) / ENTRY_TILE;
  for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int64_t t0 = t * ENTRY_TILE, t1 = min(m, t0 + ENTRY_TILE);
    int64_t hint = -1;  // tiles of one block are not contiguous here
    expand_rows<ENTRY_TILE>(rowptr, n, t0, t1, rows, scan_tmp, hint);
    for (int k = threadIdx.x; k < t1 - t0; k += OR_THREADS) src[t0 + k] = rows[rslot((int)k)];
    __syncthreads();
  }
}

__global__ void indeg_kernel(const int32_t *__restrict__ col, int64_t n, int64_t m, int32_t *__restrict__ indeg) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v = col[e];
    if (v >= 0 && v < n) atomicAdd(indeg + v, 1);
  }
}

tc_status launch_indeg(tc_ctx *ctx, const int32_t *col, int64_t n, int64_t m, int32_t *indeg) {
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(indeg, 0, sizeof(int32_t) * (size_t)n, ctx->stream));
  if (m <= 0) return TC_OK;
  indeg_kernel<<<grid_for(ctx, m, ENTRY_TILE, 8), OR_THREADS, 0, ctx->stream>>>(col, n, m, indeg);
  TC_CHECK_LAUNCH(ctx);
  return TC_OK;
}

// out[i] = rowptr[i] - shift: row pointers of a row range counted in place,
// relative to the range's first entry (tc_count_dag_range).
__global__ void shift_rowptr_kernel(const int64_t *__restrict__ rowptr, int64_t n, int64_t shift,
                                    int64_t *__restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = rowptr[i] - shift;
}

tc_status launch_shift_rowptr(tc_ctx *ctx, const int64_t *rowptr, int64_t n, int64_t shift, int64_t *out) {
  shift_rowptr_kernel<<<grid_for(ctx, n + 1, 256, 8), 256, 0, ctx->stream>>>(rowptr, n, shift, out);
  TC_CHECK_LAUNCH(ctx);
  return TC_OK;
}

tc_status launch_expand_src(tc_ctx *ctx, const int64_t *rowptr, int64_t n, int64_t m, int32_t *src) {
  if (m <= 0) return TC_OK;
  expand_src_kernel<<<grid_for(ctx, m, ENTRY_TILE, 8), OR_THREADS, 0, ctx->stream>>>(rowptr, n, m, src);
  TC_CHECK_LAUNCH(ctx);
  return TC_OK;
}

}  // namespace tc
