// Stable LSD radix sort of uint64 keys (8-bit digits, optional uint32
// payload) and an exclusive int64 scan, both "reduce then scan" over a grid
// of contiguous per-block chunks so that no block ever waits on another.
//
// Per digit pass: (1) every block histograms its chunk, (2) one block scans
// the [256 digits x G blocks] table into global offsets, (3) every block
// re-reads its chunk tile by tile, ranks items stably inside each warp with
// __match_any_sync and scatters them.  Stability: a block's chunk precedes
// the next block's chunk, warps own consecutive 256-item runs of a tile and
// lanes own consecutive items of a round.
#include <stdarg.h>

#include "dev_common.cuh"

namespace tc {

tc_status set_error(tc_ctx *ctx, tc_status st, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx) snprintf(ctx->err, sizeof(ctx->err), "%s", buf);
  set_global_error("%s", buf);
  return st;
}

tc_status arena_reserve(tc_ctx *ctx, size_t bytes) {
  ctx->arena_used = 0;
  if (bytes <= ctx->arena_cap) return TC_OK;
  if (ctx->arena) {
    TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    TC_CHECK_CUDA(ctx, cudaFree(ctx->arena));
    ctx->arena = nullptr;
    ctx->arena_cap = 0;
  }
  size_t cap = align_up(bytes + bytes / 8, size_t(1) << 20);
  cudaError_t e = cudaMalloc((void **)&ctx->arena, cap);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    ctx->arena = nullptr;
    return set_error(ctx, TC_ERR_OOM, "device arena of %zu bytes: %s", cap, cudaGetErrorString(e));
  }
  ctx->arena_cap = cap;
  return TC_OK;
}

int grid_for(const tc_ctx *ctx, int64_t items, int per_block, int blocks_per_sm) {
  int64_t want = (items + per_block - 1) / per_block;
  int64_t cap = (int64_t)ctx->num_sms * blocks_per_sm;
  if (want > cap) want = cap;
  if (want < 1) want = 1;
  return (int)want;
}

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_IPL = 8;                         // items per lane per tile
constexpr int RS_TILE = RS_THREADS * RS_IPL;      // 2048 items
constexpr int RS_BLOCKS_PER_SM = 4;

struct RsGeom {
  int G;
  int64_t chunk;
};

static RsGeom rs_geom(const tc_ctx *ctx, int64_t N) {
  RsGeom g;
  int64_t tiles = (N + RS_TILE - 1) / RS_TILE;
  int64_t G = (int64_t)ctx->num_sms * RS_BLOCKS_PER_SM;
  if (G > tiles) G = tiles;
  if (G < 1) G = 1;
  int64_t tiles_per = (tiles + G - 1) / G;
  g.chunk = tiles_per * RS_TILE;
  g.G = (int)((N + g.chunk - 1) / g.chunk);
  if (g.G < 1) g.G = 1;
  return g;
}

size_t radix_sort_scratch_bytes(const tc_ctx *ctx, int64_t N) {
  RsGeom g = rs_geom(ctx, N);
  return align_up((size_t)256 * g.G * sizeof(uint32_t), 256) + align_up((size_t)256 * g.G * sizeof(uint64_t), 256);
}

__global__ void __launch_bounds__(RS_THREADS) rs_hist_kernel(const uint64_t *__restrict__ keys, int64_t N, int shift,
                                                            int64_t chunk, uint32_t *__restrict__ hist, int G) {
  __shared__ uint32_t cnt[RS_WARPS][256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < RS_WARPS * 256; i += RS_THREADS) (&cnt[0][0])[i] = 0;
  __syncthreads();
  const int64_t b = (int64_t)blockIdx.x * chunk;
  const int64_t e = min(N, b + chunk);
  for (int64_t base = b; base < e; base += RS_THREADS) {
    const int64_t i = base + threadIdx.x;
    const bool valid = i < e;
    const unsigned vmask = __ballot_sync(TC_FULL_MASK, valid);
    if (valid) {
      const unsigned d = (unsigned)((keys[i] >> shift) & 255u);
      const unsigned peers = __match_any_sync(vmask, d);
      if (lane == __ffs(peers) - 1) cnt[warp][d] += __popc(peers);
    }
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += RS_THREADS) {
    uint32_t s = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) s += cnt[w][d];
    hist[(int64_t)blockIdx.x * 256 + d] = s;
  }
}

// Digit offsets from the block-major histogram hist[b][d]: offs[b][d] =
// (keys with a smaller digit) + (keys with digit d in blocks before b).  One
// block: 4 threads per digit, each owning a quarter of the blocks; reads are
// coalesced across digits.
__global__ void __launch_bounds__(1024) rs_scan_kernel(const uint32_t *__restrict__ hist, uint64_t *__restrict__ offs,
                                                      int G) {
  __shared__ unsigned long long part[4][256];
  __shared__ unsigned long long base[256];
  __shared__ unsigned long long tmp[33];
  const int d = threadIdx.x & 255, q = threadIdx.x >> 8;
  const int per = (G + 3) / 4;
  const int b0 = q * per, b1 = min(G, b0 + per);
  unsigned long long s = 0;
  for (int b = b0; b < b1; ++b) s += hist[(int64_t)b * 256 + d];
  part[q][d] = s;
  __syncthreads();
  unsigned long long dtot = 0;
  if (threadIdx.x < 256) dtot = part[0][d] + part[1][d] + part[2][d] + part[3][d];
  // exclusive scan of the 256 digit totals (threads 0..255; the rest add 0)
  unsigned long long tot;
  const unsigned long long ex = block_exclusive_scan<unsigned long long>(dtot, tmp, &tot);
  if (threadIdx.x < 256) base[d] = ex;
  __syncthreads();
  unsigned long long run = base[d];
  for (int k = 0; k < q; ++k) run += part[k][d];
  for (int b = b0; b < b1; ++b) {
    offs[(int64_t)b * 256 + d] = run;
    run += hist[(int64_t)b * 256 + d];
  }
}

template <bool HAS_VALS>
__global__ void __launch_bounds__(RS_THREADS) rs_scatter_kernel(const uint64_t *__restrict__ kin,
                                                               const uint32_t *__restrict__ vin,
                                                               uint64_t *__restrict__ kout,
                                                               uint32_t *__restrict__ vout, int64_t N, int shift,
                                                               int64_t chunk, const uint64_t *__restrict__ offs,
                                                               int G) {
  __shared__ uint32_t wcnt[RS_WARPS][256];
  __shared__ unsigned long long boff[256];
  __shared__ uint32_t tcnt[256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = lanemask_lt();
  for (int d = threadIdx.x; d < 256; d += RS_THREADS) boff[d] = offs[(int64_t)blockIdx.x * 256 + d];
  for (int i = threadIdx.x; i < RS_WARPS * 256; i += RS_THREADS) (&wcnt[0][0])[i] = 0;
  __syncthreads();
  const int64_t b = (int64_t)blockIdx.x * chunk;
  const int64_t e = min(N, b + chunk);
  for (int64_t t0 = b; t0 < e; t0 += RS_TILE) {
    uint64_t k[RS_IPL];
    uint32_t v[RS_IPL];
    uint32_t r[RS_IPL];
    const int64_t base = t0 + (int64_t)warp * (32 * RS_IPL);
#pragma unroll
    for (int it = 0; it < RS_IPL; ++it) {
      const int64_t idx = base + it * 32 + lane;
      const bool valid = idx < e;
      const unsigned vmask = __ballot_sync(TC_FULL_MASK, valid);
      k[it] = 0;
      v[it] = 0;
      r[it] = 0;
      if (valid) {
        k[it] = kin[idx];
        if (HAS_VALS) v[it] = vin[idx];
        const unsigned d = (unsigned)((k[it] >> shift) & 255u);
        const unsigned peers = __match_any_sync(vmask, d);
        const uint32_t before = wcnt[warp][d];
        r[it] = before + __popc(peers & lt);
        __syncwarp(vmask);
        if (lane == __ffs(peers) - 1) wcnt[warp][d] = before + __popc(peers);
        __syncwarp(vmask);
      }
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += RS_THREADS) {
      uint32_t run = 0;
#pragma unroll
      for (int w = 0; w < RS_WARPS; ++w) {
        const uint32_t c = wcnt[w][d];
        wcnt[w][d] = run;
        run += c;
      }
      tcnt[d] = run;
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < RS_IPL; ++it) {
      const int64_t idx = base + it * 32 + lane;
      if (idx < e) {
        const unsigned d = (unsigned)((k[it] >> shift) & 255u);
        const unsigned long long pos = boff[d] + wcnt[warp][d] + r[it];
        kout[pos] = k[it];
        if (HAS_VALS) vout[pos] = v[it];
      }
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += RS_THREADS) {
      boff[d] += tcnt[d];
#pragma unroll
      for (int w = 0; w < RS_WARPS; ++w) wcnt[w][d] = 0;
    }
    __syncthreads();
  }
}

tc_status radix_sort(tc_ctx *ctx, uint64_t *k0, uint64_t *k1, uint32_t *v0, uint32_t *v1, int64_t N, int begin_bit,
                     int end_bit, void *scratch, uint64_t **kres, uint32_t **vres) {
  *kres = k0;
  if (vres) *vres = v0;
  if (N <= 1 || end_bit <= begin_bit) return TC_OK;
  RsGeom g = rs_geom(ctx, N);
  uint32_t *hist = (uint32_t *)scratch;
  uint64_t *offs = (uint64_t *)((char *)scratch + align_up((size_t)256 * g.G * sizeof(uint32_t), 256));
  uint64_t *ka = k0, *kb = k1;
  uint32_t *va = v0, *vb = v1;
  const bool has_vals = v0 != nullptr;
  for (int shift = begin_bit; shift < end_bit; shift += 8) {
    rs_hist_kernel<<<g.G, RS_THREADS, 0, ctx->stream>>>(ka, N, shift, g.chunk, hist, g.G);
    TC_CHECK_LAUNCH(ctx);
    rs_scan_kernel<<<1, 1024, 0, ctx->stream>>>(hist, offs, g.G);
    TC_CHECK_LAUNCH(ctx);
    if (has_vals)
      rs_scatter_kernel<true><<<g.G, RS_THREADS, 0, ctx->stream>>>(ka, va, kb, vb, N, shift, g.chunk, offs, g.G);
    else
      rs_scatter_kernel<false><<<g.G, RS_THREADS, 0, ctx->stream>>>(ka, nullptr, kb, nullptr, N, shift, g.chunk,
                                                                    offs, g.G);
    TC_CHECK_LAUNCH(ctx);
    uint64_t *tk = ka; ka = kb; kb = tk;
    uint32_t *tv = va; va = vb; vb = tv;
  }
  *kres = ka;
  if (vres) *vres = va;
  return TC_OK;
}

// ---- exclusive scan of int64 ------------------------------------------------------

constexpr int SC_THREADS = 256;
constexpr int SC_IPT = 8;
constexpr int SC_TILE = SC_THREADS * SC_IPT;

static RsGeom sc_geom(const tc_ctx *ctx, int64_t N) {
  RsGeom g;
  int64_t tiles = (N + SC_TILE - 1) / SC_TILE;
  int64_t G = (int64_t)ctx->num_sms * 4;
  if (G > tiles) G = tiles;
  if (G < 1) G = 1;
  g.chunk = ((tiles + G - 1) / G) * SC_TILE;
  g.G = (int)((N + g.chunk - 1) / g.chunk);
  if (g.G < 1) g.G = 1;
  return g;
}

size_t scan_scratch_bytes(const tc_ctx *ctx, int64_t N) {
  RsGeom g = sc_geom(ctx, N);
  return align_up((size_t)(g.G + 1) * sizeof(int64_t), 256);
}

template <typename T>
__global__ void __launch_bounds__(SC_THREADS) sc_reduce_kernel(const T *__restrict__ in, int64_t N,
                                                              int64_t chunk, int64_t *__restrict__ sums) {
  __shared__ long long tmp[33];
  const int64_t b = (int64_t)blockIdx.x * chunk, e = min(N, b + chunk);
  long long s = 0;
  for (int64_t i = b + threadIdx.x; i < e; i += SC_THREADS) s += in[i];
  long long tot;
  block_exclusive_scan<long long>(s, tmp, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) sc_top_kernel(int64_t *sums, int G, int64_t *d_total_out) {
  __shared__ long long tmp[33];
  // G <= 4 * SMs: at most a few items per thread
  const int per = (G + blockDim.x - 1) / blockDim.x;
  const int b = threadIdx.x * per, e = min(G, b + per);
  long long s = 0;
  for (int i = b; i < e; ++i) s += sums[i];
  long long tot;
  long long run = block_exclusive_scan<long long>(s, tmp, &tot);
  for (int i = b; i < e; ++i) {
    long long t = sums[i];
    sums[i] = run;
    run += t;
  }
  if (threadIdx.x == 0) {
    sums[G] = tot;
    if (d_total_out) *d_total_out = tot;
  }
}

template <typename T>
__global__ void __launch_bounds__(SC_THREADS) sc_down_kernel(const T *in, T *out, int64_t N,
                                                            int64_t chunk, const int64_t *__restrict__ sums) {
  __shared__ long long tmp[33];
  const int64_t b = (int64_t)blockIdx.x * chunk, e = min(N, b + chunk);
  long long carry = sums[blockIdx.x];
  for (int64_t t0 = b; t0 < e; t0 += SC_TILE) {
    long long x[SC_IPT];
    long long s = 0;
    const int64_t my = t0 + (int64_t)threadIdx.x * SC_IPT;
#pragma unroll
    for (int k = 0; k < SC_IPT; ++k) {
      x[k] = (my + k < e) ? in[my + k] : 0;
      s += x[k];
    }
    long long tot;
    long long run = carry + block_exclusive_scan<long long>(s, tmp, &tot);
#pragma unroll
    for (int k = 0; k < SC_IPT; ++k) {
      if (my + k < e) out[my + k] = (T)run;
      run += x[k];
    }
    carry += tot;
  }
}

tc_status exclusive_scan_i64(tc_ctx *ctx, const int64_t *in, int64_t *out, int64_t N, void *scratch,
                             int64_t *d_total_out) {
  if (N <= 0) return TC_OK;
  RsGeom g = sc_geom(ctx, N);
  int64_t *sums = (int64_t *)scratch;
  sc_reduce_kernel<int64_t><<<g.G, SC_THREADS, 0, ctx->stream>>>(in, N, g.chunk, sums);
  TC_CHECK_LAUNCH(ctx);
  sc_top_kernel<<<1, 1024, 0, ctx->stream>>>(sums, g.G, d_total_out);
  TC_CHECK_LAUNCH(ctx);
  sc_down_kernel<int64_t><<<g.G, SC_THREADS, 0, ctx->stream>>>(in, out, N, g.chunk, sums);
  TC_CHECK_LAUNCH(ctx);
  return TC_OK;
}

tc_status exclusive_scan_u32(tc_ctx *ctx, const uint32_t *in, uint32_t *out, int64_t N, void *scratch) {
  if (N <= 0) return TC_OK;
  RsGeom g = sc_geom(ctx, N);
  int64_t *sums = (int64_t *)scratch;
  sc_reduce_kernel<uint32_t><<<g.G, SC_THREADS, 0, ctx->stream>>>(in, N, g.chunk, sums);
  TC_CHECK_LAUNCH(ctx);
  sc_top_kernel<<<1, 1024, 0, ctx->stream>>>(sums, g.G, nullptr);
  TC_CHECK_LAUNCH(ctx);
  sc_down_kernel<uint32_t><<<g.G, SC_THREADS, 0, ctx->stream>>>(in, out, N, g.chunk, sums);
  TC_CHECK_LAUNCH(ctx);
  return TC_OK;
}

}  // namespace tc
