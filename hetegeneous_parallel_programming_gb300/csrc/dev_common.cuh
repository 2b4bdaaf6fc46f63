// Device-side building blocks shared by the engine's .cu files: the ctx
// struct, error plumbing, the grow-only device arena and block/warp
// primitives (scans, row expansion of CSR tiles).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "tc_internal.h"

#define TC_FULL_MASK 0xffffffffu

constexpr int TC_MAX_PIECES = 8;

struct tc_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  // grow-only arena
  char *arena = nullptr;
  size_t arena_cap = 0;
  size_t arena_used = 0;
  // grow-only buffer for a CSR built inside a call (tc_count_edges), kept
  // apart from the arena that the count then reuses
  char *aux = nullptr;
  size_t aux_cap = 0;
  // small always-resident device state
  unsigned long long *d_total = nullptr;  // [1] running total
  unsigned int *d_flags = nullptr;        // [8] error flags / counters
  unsigned int *d_heads = nullptr;        // [64] work-queue heads
  unsigned long long *h_pinned = nullptr; // [64] pinned host scratch
  // events: [0..8) entry-point phases, [8] plan start, [9] count start,
  // [10 + a] end of arm a's kernel, [10 + TC_NUM_ARMS] and [11 + TC_NUM_ARMS]
  // around the PULL arm's probing kernel (pull_kernel) alone
  cudaEvent_t ev[12 + TC_NUM_ARMS] = {};
  bool pull_timed = false;                // the pull_kernel events belong to this call
  // host input of tc_count: the column array is uploaded in pieces on a
  // second stream while the orientation starts (one event per piece)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t piece_ev[TC_MAX_PIECES] = {};
  // learned selector
  float *d_mlp = nullptr;                 // TC_MLP_PARAM_COUNT floats
  float mlp_margin = 0.f;                 // log2-cost gain a learned switch away from the fixed arm needs
  bool mlp_loaded = false;
  // per-arm kernel occupancy (blocks per SM), filled at create
  int arm_blocks_per_sm[TC_NUM_ARMS] = {};
  int arm_units_per_sm[TC_NUM_ARMS] = {};   // independent workers (warps or blocks) per SM
  int64_t launches = 0;                   // kernels launched by the current call
  // PULL work chunks (grouped entries a warp takes at a time): largest and
  // smallest; tc_set_pull_chunks / tc_autotune_pull change them
  int pull_item = 512;
  int pull_item_min = 128;
  // tc_tuning: PULL source-block size (tiles), dense-edge ratio, and the
  // orientation passes' entry-chunk geometry (blocks per SM)
  int pull_block_tiles = 2560;
  int pull_dense_num = 1, pull_dense_den = 1;
  int orient_blocks_per_sm = 6;
  // captured back half of the batched pipeline (batch.cu), keyed by shape,
  // options and the buffers it reads
  cudaGraphExec_t batch_exec = nullptr;
  int64_t batch_key[14] = {};
  int64_t batch_launches = 0;
  // captured front half (group ids, validation, ranks, kept counts, scans)
  cudaGraphExec_t batch_front_exec = nullptr;
  int64_t batch_front_key[12] = {};
  int64_t batch_front_launches = 0;
  char err[1024] = {0};
};

namespace tc {

tc_status set_error(tc_ctx *ctx, tc_status st, const char *fmt, ...);

#define TC_CHECK_CUDA(ctx, call)                                                                \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      return ::tc::set_error((ctx), e_ == cudaErrorMemoryAllocation ? TC_ERR_OOM : TC_ERR_CUDA, \
                             "%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
  } while (0)

#define TC_CHECK_LAUNCH(ctx)                \
  do {                                      \
    (ctx)->launches++;                      \
    TC_CHECK_CUDA((ctx), cudaGetLastError()); \
  } while (0)

#define TC_TRY(expr)                  \
  do {                                \
    tc_status s_ = (expr);            \
    if (s_ != TC_OK) return s_;       \
  } while (0)

// Make sure the arena holds at least `bytes`; resets the bump pointer.
tc_status arena_reserve(tc_ctx *ctx, size_t bytes);

static inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Bump allocation inside a reserved arena (256-byte aligned).
struct Bump {
  char *base;
  size_t cap, used = 0;
  bool overflow = false;
  template <typename T>
  T *take(int64_t count) {
    size_t bytes = align_up((size_t)(count > 0 ? count : 1) * sizeof(T), 256);
    if (used + bytes > cap) { overflow = true; return nullptr; }
    T *p = reinterpret_cast<T *>(base + used);
    used += bytes;
    return p;
  }
};

// Size accounting twin of Bump (same rounding).
struct Sizer {
  size_t used = 0;
  template <typename T>
  void take(int64_t count) { used += align_up((size_t)(count > 0 ? count : 1) * sizeof(T), 256); }
};

// ---- device primitives ------------------------------------------------------

// Bulk asynchronous copies (the TMA unit, non-tensor form) with mbarrier
// completion.  A copy moves `bytes` (a multiple of 16) from a 16-byte
// aligned global address to a 16-byte aligned shared address and completes
// the mbarrier's transaction count; waits poll try_wait with a bound.
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes mbarrier initialisation visible to the async (bulk copy) proxy.
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Orders this thread's earlier generic shared-memory accesses before later
// async-proxy accesses (a bulk copy overwriting a buffer that was read).
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// Bulk prefetch of [src, src + bytes) into L2 (no registers held, no
// completion to wait for): src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_prefetch_l2(const void *src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// True once the mbarrier phase of the given parity has completed.
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Polls at most `limit` times; false when the phase did not complete.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(TC_FULL_MASK, v, o);
  return v;
}

// Exclusive block scan of one value per thread (blockDim.x a multiple of 32,
// at most 1024).  `tmp` is shared scratch of >= 32 entries.  Returns the
// thread's exclusive prefix; *total receives the block sum.
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T *tmp, T *total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(TC_FULL_MASK, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) tmp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = lane < nw ? tmp[lane] : T(0);
    T wx = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(TC_FULL_MASK, wx, o);
      if (lane >= o) wx += y;
    }
    if (lane < nw) tmp[lane] = wx - w;
    if (lane == nw - 1) tmp[32] = wx;
  }
  __syncthreads();
  T res = tmp[warp] + x - v;
  *total = tmp[32];
  __syncthreads();
  return res;
}

// First row r with rowptr[r+1] > e (the row holding entry e), for a
// monotone rowptr of n+1 entries and 0 <= e < rowptr[n].
__device__ __forceinline__ int64_t row_of_entry(const int64_t *__restrict__ rowptr, int64_t n, int64_t e) {
  int64_t lo = 0, hi = n;  // answer in [0, n)
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (rowptr[mid] <= e) lo = mid; else hi = mid;
  }
  return lo;
}

// Shared row array of an entry tile: entry i sits in slot i + i / 32 (one
// pad word per 32 entries), so the max-scan below, where thread t walks
// entries [8t, 8t + 8), hits 32 distinct banks at every step (without the
// pad it is 8-way conflicted), while 32 consecutive entries read by a warp
// stay in 32 consecutive slots.
template <int TILE>
constexpr int row_slots() { return TILE + TILE / 32; }
__device__ __forceinline__ int rslot(int i) { return i + (i >> 5); }

// Row of every entry of the tile [t0, t_end) of a CSR, into rows[rslot(0 ..
// t_end-t0-1)] (shared, row_slots<TILE>() slots).  All threads of the block call it with the same
// `hint`: -1, or the row of entry t0 - 1 (the previous tile's last entry),
// which it updates to the row of entry t_end - 1.  With a hint one warp finds
// the tile's first row among the next 32 rows instead of a binary search over
// rowptr.  Ends synchronised.
template <int TILE>
__device__ void expand_rows(const int64_t *__restrict__ rowptr, int64_t n, int64_t t0, int64_t t_end,
                            int *rows, int *scan_tmp, int64_t &hint) {
  __shared__ int64_t s_first;
  for (int i = threadIdx.x; i < TILE; i += blockDim.x) rows[rslot(i)] = -1;
  if (threadIdx.x < 32) {
    int64_t r = -1;
    if (hint >= 0) {  // first r >= hint with rowptr[r + 1] > t0
      const int64_t rr = hint + threadIdx.x;
      const unsigned bal = __ballot_sync(TC_FULL_MASK, rr < n && rowptr[rr + 1] > t0);
      if (bal) r = hint + __ffs(bal) - 1;
    }
    if (r < 0) r = row_of_entry(rowptr, n, t0);
    if (threadIdx.x == 0) s_first = r;
  }
  __syncthreads();
  const int64_t r0 = s_first;
  if (threadIdx.x == 0) rows[rslot(0)] = (int)r0;
  for (int64_t r = r0 + 1 + threadIdx.x; r < n; r += blockDim.x) {
    const int64_t s = rowptr[r];
    if (s >= t_end) break;
    if (s > t0) atomicMax(&rows[rslot((int)(s - t0))], (int)r);
  }
  __syncthreads();
  // inclusive max-scan (row ids only grow): per-thread segment, then block.
  constexpr int PER = TILE / 256;  // callers use 256 threads
  int base = threadIdx.x * PER;
  int m = -1;
#pragma unroll
  for (int k = 0; k < PER; ++k) m = max(m, rows[rslot(base + k)]);
  // exclusive max-scan of m across the block
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = m;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(TC_FULL_MASK, x, o);
    if (lane >= o) x = max(x, y);
  }
  if (lane == 31) scan_tmp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = lane < (int)(blockDim.x >> 5) ? scan_tmp[lane] : -1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(TC_FULL_MASK, w, o);
      if (lane >= o) w = max(w, y);
    }
    scan_tmp[lane] = w;
  }
  __syncthreads();
  int carry = warp > 0 ? scan_tmp[warp - 1] : -1;
  int xin = __shfl_up_sync(TC_FULL_MASK, x, 1);
  if (lane > 0) carry = max(carry, xin);
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    carry = max(carry, rows[rslot(base + k)]);
    rows[rslot(base + k)] = carry;
  }
  __syncthreads();
  hint = rows[rslot((int)(t_end - t0 - 1))];
}

// ---- host-side launch helpers shared by the .cu files --------------------------

// Radix sort (radix_sort.cu): stable LSD sort of uint64 keys on bits
// [begin_bit, end_bit), optional uint32 payload.  k0/v0 hold the input;
// k1/v1 are same-sized scratch.  On return *kres / *vres point at the sorted
// data.
size_t radix_sort_scratch_bytes(const tc_ctx *ctx, int64_t N);
tc_status radix_sort(tc_ctx *ctx, uint64_t *k0, uint64_t *k1, uint32_t *v0, uint32_t *v1, int64_t N, int begin_bit,
                     int end_bit, void *scratch, uint64_t **kres, uint32_t **vres);

// Exclusive scan of int64 values (scan.cu helpers in radix_sort.cu).
size_t scan_scratch_bytes(const tc_ctx *ctx, int64_t N);
// 32-bit counts whose total stays below 2^32 (scratch as for the int64 scan)
tc_status exclusive_scan_u32(tc_ctx *ctx, const uint32_t *in, uint32_t *out, int64_t N, void *scratch);
tc_status exclusive_scan_i64(tc_ctx *ctx, const int64_t *in, int64_t *out, int64_t N, void *scratch,
                             int64_t *d_total_out);

int grid_for(const tc_ctx *ctx, int64_t items, int per_block, int blocks_per_sm);

}  // namespace tc
