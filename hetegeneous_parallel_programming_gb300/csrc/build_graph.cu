// Device-side graph construction: seeded edge generators (bit-identical to
// the host generators) and the symmetric CSR builder (symmetrise, drop self
// loops, sort, dedup) that turns edge samples into the clean GraphMiner-style
// CSR the counting path expects.
#include <algorithm>
#include <vector>

#include "engine.cuh"
#include "tc_gen_common.h"

using namespace tc;

namespace tc {

__global__ void gen_er_kernel(uint64_t key, uint64_t n, int64_t M, int32_t *src, int32_t *dst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x)
    tc_er_sample(key, n, (uint64_t)i, &src[i], &dst[i]);
}

__global__ void gen_rmat_kernel(uint64_t key, int scale, uint64_t t1, uint64_t t2, uint64_t t3, int64_t M,
                                int32_t *src, int32_t *dst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x)
    tc_rmat_sample(key, scale, t1, t2, t3, (uint64_t)i, &src[i], &dst[i]);
}

__global__ void gen_cl_kernel(uint64_t key, const uint64_t *cum, int64_t n, int64_t M, int32_t *src, int32_t *dst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x)
    tc_cl_sample(key, cum, n, (uint64_t)i, &src[i], &dst[i]);
}

// Two directed keys per undirected sample; self loops and bad ids become the
// all-ones sentinel, which sorts after every real key.
__global__ void edge_keys_kernel(const int32_t *__restrict__ src, const int32_t *__restrict__ dst, int64_t M,
                                 int64_t n, int bits, uint64_t *__restrict__ keys) {
  const uint64_t sentinel = (bits >= 32) ? ~0ULL : ((1ULL << (2 * bits)) - 1);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t u = src[i], v = dst[i];
    if (u == v || u < 0 || v < 0 || (int64_t)u >= n || (int64_t)v >= n) {
      keys[2 * i] = sentinel;
      keys[2 * i + 1] = sentinel;
    } else {
      keys[2 * i] = ((uint64_t)u << bits) | (uint64_t)v;
      keys[2 * i + 1] = ((uint64_t)v << bits) | (uint64_t)u;
    }
  }
}

__global__ void unique_flag_kernel(const uint64_t *__restrict__ keys, int64_t N, uint64_t sentinel,
                                   int64_t *__restrict__ flag) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[i];
    flag[i] = (k != sentinel && (i == 0 || keys[i - 1] != k)) ? 1 : 0;
  }
}

__global__ void unique_scatter_kernel(const uint64_t *__restrict__ keys, const int64_t *__restrict__ pos, int64_t N,
                                      uint64_t sentinel, int bits, int32_t *__restrict__ col,
                                      unsigned long long *__restrict__ deg) {
  const uint64_t mask = (1ULL << bits) - 1;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[i];
    if (k != sentinel && (i == 0 || keys[i - 1] != k)) {
      col[pos[i]] = (int32_t)(k & mask);
      atomicAdd(&deg[k >> bits], 1ULL);
    }
  }
}

}  // namespace tc

extern "C" {

tc_status tc_gen_edges_device(tc_ctx *ctx, const tc_gen_params *p, int32_t *src, int32_t *dst, int64_t capacity,
                              int64_t *count_out) {
  if (!ctx || !p || !count_out) return set_error(ctx, TC_ERR_INVALID_ARG, "null argument");
  if (p->kind == TC_GEN_RGG) return set_error(ctx, TC_ERR_UNSUPPORTED, "RGG is generated on the host only");
  const int64_t M = tc_gen_num_samples(p);
  if (M < 0) return set_error(ctx, TC_ERR_INVALID_ARG, "%s", global_error());
  *count_out = M;
  if (!src || !dst || M > capacity)
    return set_error(ctx, TC_ERR_INVALID_ARG, "edge buffers hold %lld samples, %lld needed", (long long)capacity,
                     (long long)M);
  TC_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  const int grid = ctx->num_sms * 8;
  if (p->kind == TC_GEN_ER) {
    if (p->n < 1 || p->n > 2147483647LL) return set_error(ctx, TC_ERR_INVALID_ARG, "bad n");
    gen_er_kernel<<<grid, 256, 0, ctx->stream>>>(tc_stream_key(p->seed, TC_SID_ER), (uint64_t)p->n, M, src, dst);
  } else if (p->kind == TC_GEN_RMAT) {
    if (p->scale < 1 || p->scale > 30) return set_error(ctx, TC_ERR_INVALID_ARG, "bad RMAT scale");
    uint64_t t1, t2, t3;
    rmat_thresholds(p->a, p->b, p->c, &t1, &t2, &t3);
    gen_rmat_kernel<<<grid, 256, 0, ctx->stream>>>(tc_stream_key(p->seed, TC_SID_RMAT), p->scale, t1, t2, t3, M, src,
                                                   dst);
  } else if (p->kind == TC_GEN_CHUNG_LU) {
    if (p->n < 1 || p->n > 2147483647LL || !(p->gamma > 1.0)) return set_error(ctx, TC_ERR_INVALID_ARG, "bad CL");
    std::vector<uint64_t> cum((size_t)p->n);
    chung_lu_table(p->n, p->avg_degree, p->gamma, cum.data());
    TC_TRY(arena_reserve(ctx, sizeof(uint64_t) * (size_t)p->n));
    uint64_t *d_cum = (uint64_t *)ctx->arena;
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(d_cum, cum.data(), sizeof(uint64_t) * (size_t)p->n, cudaMemcpyHostToDevice,
                                       ctx->stream));
    gen_cl_kernel<<<grid, 256, 0, ctx->stream>>>(tc_stream_key(p->seed, TC_SID_CL), d_cum, p->n, M, src, dst);
    TC_CHECK_CUDA(ctx, cudaGetLastError());
    TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // cum is read from pageable memory above
    return TC_OK;
  } else {
    return set_error(ctx, TC_ERR_INVALID_ARG, "unknown generator %d", p->kind);
  }
  TC_CHECK_CUDA(ctx, cudaGetLastError());
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TC_OK;
}

tc_status tc_csr_from_edges(tc_ctx *ctx, int64_t n, int64_t M, const int32_t *src, const int32_t *dst,
                            int32_t on_device, int64_t *rowptr, int32_t *colidx, int64_t capacity, int64_t *nnz_out) {
  if (!ctx || !rowptr || !nnz_out || (M > 0 && (!src || !dst)) || M < 0)
    return set_error(ctx, TC_ERR_INVALID_ARG, "null argument");
  if (n < 1 || n > 2147483647LL) return set_error(ctx, TC_ERR_UNSUPPORTED, "n outside [1, 2^31-1]");
  if (2 * M >= (int64_t(1) << 32)) return set_error(ctx, TC_ERR_UNSUPPORTED, "too many edge samples");
  TC_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  const int bits = bit_width_u64(n > 1 ? (uint64_t)(n - 1) : 1);
  const uint64_t sentinel = (1ULL << (2 * bits)) - 1;
  const int64_t N = 2 * M;
  Sizer sz;
  if (!on_device) { sz.take<int32_t>(M); sz.take<int32_t>(M); }
  sz.take<uint64_t>(N); sz.take<uint64_t>(N);
  sz.take<int64_t>(N);
  sz.take<int64_t>(n + 1);
  sz.take<char>((int64_t)std::max(radix_sort_scratch_bytes(ctx, std::max<int64_t>(N, 1)),
                                  scan_scratch_bytes(ctx, std::max<int64_t>(N, n + 1))));
  if (!on_device) { sz.take<int64_t>(n + 1); sz.take<int32_t>(N); }
  TC_TRY(arena_reserve(ctx, sz.used));
  Bump bump{ctx->arena, ctx->arena_cap};
  const int32_t *dsrc = src, *ddst = dst;
  if (!on_device) {
    int32_t *s = bump.take<int32_t>(M), *d = bump.take<int32_t>(M);
    if (M > 0) {
      TC_CHECK_CUDA(ctx, cudaMemcpyAsync(s, src, sizeof(int32_t) * M, cudaMemcpyHostToDevice, ctx->stream));
      TC_CHECK_CUDA(ctx, cudaMemcpyAsync(d, dst, sizeof(int32_t) * M, cudaMemcpyHostToDevice, ctx->stream));
    }
    dsrc = s;
    ddst = d;
  }
  uint64_t *k0 = bump.take<uint64_t>(N), *k1 = bump.take<uint64_t>(N);
  int64_t *flag = bump.take<int64_t>(N);
  int64_t *deg = bump.take<int64_t>(n + 1);
  void *scratch = bump.take<char>((int64_t)std::max(radix_sort_scratch_bytes(ctx, std::max<int64_t>(N, 1)),
                                                    scan_scratch_bytes(ctx, std::max<int64_t>(N, n + 1))));
  int64_t *drow = on_device ? rowptr : bump.take<int64_t>(n + 1);
  int32_t *dcol_stage = on_device ? nullptr : bump.take<int32_t>(N);
  if (bump.overflow) return set_error(ctx, TC_ERR_OOM, "arena overflow");
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(deg, 0, sizeof(int64_t) * (size_t)(n + 1), ctx->stream));
  int64_t nnz = 0;
  if (M > 0) {
    edge_keys_kernel<<<grid_for(ctx, M, 256, 8), 256, 0, ctx->stream>>>(dsrc, ddst, M, n, bits, k0);
    TC_CHECK_LAUNCH(ctx);
    uint64_t *sk = nullptr;
    TC_TRY(radix_sort(ctx, k0, k1, nullptr, nullptr, N, 0, 2 * bits, scratch, &sk, nullptr));
    unique_flag_kernel<<<grid_for(ctx, N, 256, 8), 256, 0, ctx->stream>>>(sk, N, sentinel, flag);
    TC_CHECK_LAUNCH(ctx);
    TC_TRY(exclusive_scan_i64(ctx, flag, flag, N, scratch, (int64_t *)&ctx->d_total[0]));
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ctx->h_pinned[0], ctx->d_total, sizeof(int64_t), cudaMemcpyDeviceToHost,
                                       ctx->stream));
    TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    nnz = (int64_t)ctx->h_pinned[0];
    *nnz_out = nnz;
    if (nnz > capacity || !colidx)
      return set_error(ctx, TC_ERR_INVALID_ARG, "colidx holds %lld entries, %lld needed", (long long)capacity,
                       (long long)nnz);
    int32_t *dcol = on_device ? colidx : dcol_stage;
    unique_scatter_kernel<<<grid_for(ctx, N, 256, 8), 256, 0, ctx->stream>>>(sk, flag, N, sentinel, bits, dcol,
                                                                             (unsigned long long *)deg);
    TC_CHECK_LAUNCH(ctx);
    if (!on_device && nnz > 0)
      TC_CHECK_CUDA(ctx, cudaMemcpyAsync(colidx, dcol_stage, sizeof(int32_t) * nnz, cudaMemcpyDeviceToHost,
                                         ctx->stream));
  } else {
    *nnz_out = 0;
  }
  TC_TRY(exclusive_scan_i64(ctx, deg, drow, n + 1, scratch, nullptr));
  if (!on_device)
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(rowptr, drow, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TC_OK;
}

}  // extern "C"

extern "C" tc_status tc_count_edges(tc_ctx *ctx, int64_t n, int64_t M, const int32_t *src, const int32_t *dst,
                                    int32_t on_device, const tc_opts *opts, uint64_t *total, tc_stats *stats) {
  if (!ctx || !total) return set_error(ctx, TC_ERR_INVALID_ARG, "null ctx or total");
  if (n < 1 || n > 2147483647LL || M < 0 || (M > 0 && (!src || !dst)))
    return set_error(ctx, TC_ERR_INVALID_ARG, "bad n or edge list");
  if (2 * M >= (int64_t(1) << 32)) return set_error(ctx, TC_ERR_UNSUPPORTED, "too many edge samples");
  TC_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  // the built CSR lives in ctx->aux: at most 2M entries
  const size_t need = align_up(sizeof(int64_t) * (size_t)(n + 1), 256) + align_up(sizeof(int32_t) * (size_t)(2 * M + 1), 256);
  if (need > ctx->aux_cap) {
    TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->aux) TC_CHECK_CUDA(ctx, cudaFree(ctx->aux));
    ctx->aux = nullptr;
    ctx->aux_cap = 0;
    cudaError_t e = cudaMalloc((void **)&ctx->aux, need);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return set_error(ctx, TC_ERR_OOM, "edge-list CSR buffer of %zu bytes: %s", need, cudaGetErrorString(e));
    }
    ctx->aux_cap = need;
  }
  int64_t *rowptr = (int64_t *)ctx->aux;
  int32_t *colidx = (int32_t *)(ctx->aux + align_up(sizeof(int64_t) * (size_t)(n + 1), 256));
  int64_t nnz = 0;
  TC_TRY(tc_csr_from_edges(ctx, n, M, src, dst, on_device, rowptr, colidx, 2 * M, &nnz));
  tc_csr g{n, nnz, rowptr, colidx, 1};
  return tc_count(ctx, &g, opts, total, nullptr, 0, stats);
}
