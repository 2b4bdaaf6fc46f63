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

void orient_geometry(const tc_ctx *ctx, int64_t nnz, int *G, int64_t *chunk) {
  int64_t tiles = (nnz + ENTRY_TILE - 1) / ENTRY_TILE;
  int64_t g = (int64_t)ctx->num_sms * 4;
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
  __shared__ int rows[ENTRY_TILE];
  __shared__ int scan_tmp[32];
  unsigned f = 0;
  const int64_t tiles = (nnz + ENTRY_TILE - 1) / ENTRY_TILE;
  for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int64_t t0 = t * ENTRY_TILE, t1 = min(nnz, t0 + ENTRY_TILE);
    if (simple) expand_rows<ENTRY_TILE>(rowptr, n, t0, t1, rows, scan_tmp);
#pragma unroll
    for (int k = 0; k < OR_PER; ++k) {
      const int64_t e = t0 + k * OR_THREADS + threadIdx.x;
      if (e >= t1) continue;
      const int32_t v = col[e];
      if (v < 0 || (int64_t)v >= n) { f |= VF_ID_RANGE; continue; }
      if (simple) {
        const int u = rows[e - t0];
        if (u == v) f |= VF_SELF_LOOP;
        if (u >= 0 && u < n && e > 0 && e > rowptr[u] && col[e - 1] >= v) f |= VF_UNSORTED;
      }
    }
    __syncthreads();
  }
  f = __reduce_or_sync(TC_FULL_MASK, f);
  if ((threadIdx.x & 31) == 0 && f) atomicOr(flags, f);
}

tc_status launch_validate(tc_ctx *ctx, const DevCSR &g, bool simple) {
  validate_rowptr_kernel<<<grid_for(ctx, g.n + 1, 256, 8), 256, 0, ctx->stream>>>(g.rowptr, g.n, g.nnz,
                                                                                  ctx->d_flags);
  TC_CHECK_LAUNCH(ctx);
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
__global__ void __launch_bounds__(OR_THREADS) kept_count_kernel(const int64_t *__restrict__ rowptr,
                                                               const int32_t *__restrict__ col, int64_t n,
                                                               int64_t nnz, int64_t chunk,
                                                               const int32_t *__restrict__ rank,
                                                               unsigned long long *__restrict__ kept,
                                                               int64_t *__restrict__ bcount) {
  __shared__ int rows[ENTRY_TILE];
  __shared__ int scan_tmp[32];
  __shared__ unsigned long long bsum;
  if (threadIdx.x == 0) bsum = 0;
  const int64_t b = (int64_t)blockIdx.x * chunk, e_end = min(nnz, b + chunk);
  unsigned long long mine = 0;
  const int lane = threadIdx.x & 31;
  for (int64_t t0 = b; t0 < e_end; t0 += ENTRY_TILE) {
    const int64_t t1 = min(e_end, t0 + ENTRY_TILE);
    expand_rows<ENTRY_TILE>(rowptr, n, t0, t1, rows, scan_tmp);
#pragma unroll
    for (int k = 0; k < OR_PER; ++k) {
      const int64_t e = t0 + k * OR_THREADS + threadIdx.x;
      bool keep = false;
      int u = -1;
      if (e < t1) {
        u = rows[e - t0];
        const int32_t v = col[e];
        keep = u >= 0 && v >= 0 && (int64_t)v < n && rank[v] > rank[u];
      }
      const unsigned km = __ballot_sync(TC_FULL_MASK, keep);
      if (keep) {
        const unsigned peers = __match_any_sync(km, u);
        if (lane == __ffs(peers) - 1) atomicAdd(&kept[u], (unsigned long long)__popc(peers));
      }
      mine += keep ? 1 : 0;
    }
    __syncthreads();
  }
  mine = warp_sum(mine);
  if (lane == 0 && mine) atomicAdd(&bsum, mine);
  __syncthreads();
  if (threadIdx.x == 0) bcount[blockIdx.x] = (int64_t)bsum;
}

tc_status orient_phase_a(tc_ctx *ctx, const DevCSR &g, OrientBufs &b) {
  const int bits = vertex_bits(g.n);
  orient_geometry(ctx, g.nnz, &b.G, &b.chunk);
  if (2 * bits + b.group_bits > 64)
    return set_error(ctx, TC_ERR_UNSUPPORTED, "rank key needs %d bits", 2 * bits + b.group_bits);
  deg_key_kernel<<<grid_for(ctx, g.n, 256, 8), 256, 0, ctx->stream>>>(g.rowptr, g.n, bits, b.vgroup, b.vkeys0);
  TC_CHECK_LAUNCH(ctx);
  uint64_t *sorted = nullptr;
  TC_TRY(radix_sort(ctx, b.vkeys0, b.vkeys1, nullptr, nullptr, g.n, 2 * bits + (b.vgroup ? b.group_bits : 0),
                    b.sort_scratch, &sorted, nullptr));
  rank_kernel<<<grid_for(ctx, g.n, 256, 8), 256, 0, ctx->stream>>>(sorted, g.n, (1ULL << bits) - 1, b.rank);
  TC_CHECK_LAUNCH(ctx);
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(b.kept, 0, sizeof(int64_t) * (size_t)(g.n + 1), ctx->stream));
  if (g.nnz > 0) {
    kept_count_kernel<<<b.G, OR_THREADS, 0, ctx->stream>>>(g.rowptr, g.col, g.n, g.nnz, b.chunk, b.rank,
                                                           (unsigned long long *)b.kept, b.bcount);
    TC_CHECK_LAUNCH(ctx);
    TC_TRY(exclusive_scan_i64(ctx, b.bcount, b.bcount, b.G, b.sort_scratch, b.d_m));
  } else {
    TC_CHECK_CUDA(ctx, cudaMemsetAsync(b.d_m, 0, sizeof(int64_t), ctx->stream));
  }
  return TC_OK;
}

// ---- phase B: compaction, relabel sort, DAG arrays ---------------------------

template <bool VALS, bool DAGCOL>
__global__ void __launch_bounds__(OR_THREADS) emit_kernel(const int64_t *__restrict__ rowptr,
                                                         const int32_t *__restrict__ col, int64_t n, int64_t nnz,
                                                         int64_t chunk, const int32_t *__restrict__ rank,
                                                         const int64_t *__restrict__ boff, int bits,
                                                         uint64_t *__restrict__ keys, uint32_t *__restrict__ vals,
                                                         int32_t *__restrict__ dag_col) {
  __shared__ int rows[ENTRY_TILE];
  __shared__ int scan_tmp[32];
  __shared__ long long stmp[33];
  const int64_t b = (int64_t)blockIdx.x * chunk, e_end = min(nnz, b + chunk);
  long long carry = boff[blockIdx.x];
  for (int64_t t0 = b; t0 < e_end; t0 += ENTRY_TILE) {
    const int64_t t1 = min(e_end, t0 + ENTRY_TILE);
    expand_rows<ENTRY_TILE>(rowptr, n, t0, t1, rows, scan_tmp);
    int32_t vv[OR_PER];
    int32_t ru = 0;
    unsigned keepm = 0;
    const int first = threadIdx.x * OR_PER;
#pragma unroll
    for (int k = 0; k < OR_PER; ++k) {
      const int64_t e = t0 + first + k;
      vv[k] = -1;
      if (e < t1) {
        const int u = rows[first + k];
        const int32_t v = col[e];
        if (u >= 0 && v >= 0 && (int64_t)v < n) {
          const int32_t rv = rank[v], rr = rank[u];
          if (rv > rr) {
            keepm |= 1u << k;
            vv[k] = v;
            ru = rr;  // all kept entries of one thread may span rows; recomputed below
          }
        }
      }
    }
    (void)ru;
    long long tot;
    long long pos = carry + block_exclusive_scan<long long>((long long)__popc(keepm), stmp, &tot);
#pragma unroll
    for (int k = 0; k < OR_PER; ++k) {
      if (keepm & (1u << k)) {
        const int u = rows[first + k];
        const uint64_t key = ((uint64_t)(uint32_t)rank[u] << bits) | (uint64_t)(uint32_t)rank[vv[k]];
        keys[pos] = key;
        if (VALS) vals[pos] = (uint32_t)pos;
        if (DAGCOL) dag_col[pos] = vv[k];
        ++pos;
      }
    }
    carry += tot;
    __syncthreads();
  }
}

__global__ void extract_kernel(const uint64_t *__restrict__ keys, int64_t m, int bits, int32_t *__restrict__ ncol,
                               int32_t *__restrict__ nsrc) {
  const uint64_t mask = (1ULL << bits) - 1;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[j];
    ncol[j] = (int32_t)(k & mask);
    nsrc[j] = (int32_t)(k >> bits);
  }
}

__global__ void dnew_kernel(const int64_t *__restrict__ kept, const int32_t *__restrict__ rank, int64_t n,
                            int64_t *__restrict__ dnew) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x)
    dnew[rank[u]] = kept[u];
  if (blockIdx.x == 0 && threadIdx.x == 0) dnew[n] = 0;
}

tc_status orient_phase_b(tc_ctx *ctx, const DevCSR &g, OrientBufs &b, int64_t m, bool want_perm, bool want_dag_cols,
                         DevDag *out) {
  const int bits = vertex_bits(g.n);
  if (g.nnz > 0 && m > 0) {
#define TC_EMIT(V, D)                                                                                    \
  emit_kernel<V, D><<<b.G, OR_THREADS, 0, ctx->stream>>>(g.rowptr, g.col, g.n, g.nnz, b.chunk, b.rank, b.bcount, \
                                                         bits, b.ekeys0, b.evals0, b.dag_col)
    if (want_perm && want_dag_cols) TC_EMIT(true, true);
    else if (want_perm) TC_EMIT(true, false);
    else if (want_dag_cols) TC_EMIT(false, true);
    else TC_EMIT(false, false);
#undef TC_EMIT
    TC_CHECK_LAUNCH(ctx);
  }
  uint64_t *skeys = b.ekeys0;
  uint32_t *svals = want_perm ? b.evals0 : nullptr;
  if (m > 1)
    TC_TRY(radix_sort(ctx, b.ekeys0, b.ekeys1, want_perm ? b.evals0 : nullptr, want_perm ? b.evals1 : nullptr, m,
                      2 * bits, b.sort_scratch, &skeys, want_perm ? &svals : nullptr));
  if (m > 0) {
    extract_kernel<<<grid_for(ctx, m, 256, 8), 256, 0, ctx->stream>>>(skeys, m, bits, b.ncol, b.nsrc);
    TC_CHECK_LAUNCH(ctx);
  }
  dnew_kernel<<<grid_for(ctx, g.n, 256, 8), 256, 0, ctx->stream>>>(b.kept, b.rank, g.n, b.dnew);
  TC_CHECK_LAUNCH(ctx);
  TC_TRY(exclusive_scan_i64(ctx, b.dnew, b.nrowptr, g.n + 1, b.sort_scratch, nullptr));
  out->n = g.n;
  out->m = m;
  out->rowptr = b.nrowptr;
  out->col = b.ncol;
  out->src = b.nsrc;
  out->perm = want_perm ? svals : nullptr;
  out->restrict_after = 1;
  return TC_OK;
}

// ---- row of each entry (for caller-oriented DAGs) -----------------------------

__global__ void __launch_bounds__(OR_THREADS) expand_src_kernel(const int64_t *__restrict__ rowptr, int64_t n,
                                                               int64_t m, int32_t *__restrict__ src) {
  __shared__ int rows[ENTRY_TILE];
  __shared__ int scan_tmp[32];
  const int64_t tiles = (m + ENTRY_TILE - 1) / ENTRY_TILE;
  for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int64_t t0 = t * ENTRY_TILE, t1 = min(m, t0 + ENTRY_TILE);
    expand_rows<ENTRY_TILE>(rowptr, n, t0, t1, rows, scan_tmp);
    for (int k = threadIdx.x; k < t1 - t0; k += OR_THREADS) src[t0 + k] = rows[k];
    __syncthreads();
  }
}

tc_status launch_expand_src(tc_ctx *ctx, const int64_t *rowptr, int64_t n, int64_t m, int32_t *src) {
  if (m <= 0) return TC_OK;
  expand_src_kernel<<<grid_for(ctx, m, ENTRY_TILE, 8), OR_THREADS, 0, ctx->stream>>>(rowptr, n, m, src);
  TC_CHECK_LAUNCH(ctx);
  return TC_OK;
}

}  // namespace tc
