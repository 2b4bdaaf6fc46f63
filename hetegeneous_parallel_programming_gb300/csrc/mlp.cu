// MLP cost model of the learned strategy selector: 16 tile features ->
// 64 -> 64 -> one predicted relative log-cost per arm (ReLU hidden layers).
//
// Training runs on the device with this file's kernels: a block computes the
// forward pass, the backward pass and the per-block parameter gradients of
// 32 rows (deterministic order), a second kernel sums the block partials in
// fixed order and a third applies Adam (Kingma & Ba, ICLR 2015).  Targets are
// log2 costs centred per tile (the selector only needs the argmin), and the
// loss is the mean squared error over rows and arms.
#include <cmath>
#include <vector>

#include "engine.cuh"
#include "tc_gen_common.h"

using namespace tc;

namespace tc {

constexpr int F = TC_MLP_FEATURES, H = TC_MLP_HIDDEN, K = TC_NUM_ARMS;
constexpr int P = TC_MLP_PARAM_COUNT;
constexpr int OFF_W1 = 0, OFF_B1 = F * H, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H, OFF_W3 = OFF_B2 + H,
              OFF_B3 = OFF_W3 + H * K;
static_assert(OFF_B3 + K == P, "parameter layout");
constexpr int ROWS = 32;
constexpr int MT = 256;

struct RowBuf {
  float x[ROWS][F];
  float z1[ROWS][H];
  float z2[ROWS][H];
  float dz1[ROWS][H];
  float dz2[ROWS][H];
  float dy[ROWS][K];
};

// Forward + backward of rows [r0, r0+ROWS) of the batch, per-block gradient
// partials into part[blockIdx.x][P], per-block loss into loss_part.
__global__ void __launch_bounds__(MT) mlp_fwd_bwd_kernel(const float *__restrict__ w, const float *__restrict__ X,
                                                        const float *__restrict__ Y, const int32_t *__restrict__ idx,
                                                        int64_t rows, float inv_norm, float *__restrict__ part,
                                                        float *__restrict__ loss_part) {
  extern __shared__ float smem[];
  RowBuf &b = *reinterpret_cast<RowBuf *>(smem);
  float *sw = smem + sizeof(RowBuf) / sizeof(float);
  __shared__ float s_loss[MT / 32];
  for (int i = threadIdx.x; i < P; i += MT) sw[i] = w[i];
  const int64_t r0 = (int64_t)blockIdx.x * ROWS;
  const int nr = (int)min((int64_t)ROWS, rows - r0);
  for (int i = threadIdx.x; i < ROWS * F; i += MT) {
    const int r = i / F, f = i % F;
    b.x[r][f] = r < nr ? X[(int64_t)(idx ? idx[r0 + r] : r0 + r) * F + f] : 0.f;
  }
  __syncthreads();
  // layer 1: thread (r, j) pairs
  for (int i = threadIdx.x; i < ROWS * H; i += MT) {
    const int r = i / H, j = i % H;
    float a = sw[OFF_B1 + j];
    for (int f = 0; f < F; ++f) a = fmaf(b.x[r][f], sw[OFF_W1 + f * H + j], a);
    b.z1[r][j] = a;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < ROWS * H; i += MT) {
    const int r = i / H, j = i % H;
    float a = sw[OFF_B2 + j];
    for (int q = 0; q < H; ++q) a = fmaf(fmaxf(b.z1[r][q], 0.f), sw[OFF_W2 + q * H + j], a);
    b.z2[r][j] = a;
  }
  __syncthreads();
  float lsum = 0.f;
  for (int i = threadIdx.x; i < ROWS * K; i += MT) {
    const int r = i / K, k = i % K;
    float a = sw[OFF_B3 + k];
    for (int q = 0; q < H; ++q) a = fmaf(fmaxf(b.z2[r][q], 0.f), sw[OFF_W3 + q * K + k], a);
    float d = 0.f;
    if (r < nr) {
      const float t = Y[(int64_t)(idx ? idx[r0 + r] : r0 + r) * K + k];
      d = a - t;
      lsum += 0.5f * d * d;
    }
    b.dy[r][k] = d * inv_norm;
  }
  lsum = warp_sum(lsum);
  if ((threadIdx.x & 31) == 0) s_loss[threadIdx.x >> 5] = lsum;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f;
    for (int q = 0; q < MT / 32; ++q) s += s_loss[q];
    loss_part[blockIdx.x] = s * inv_norm;
  }
  // dA2 = dY W3^T, dZ2 = dA2 * (Z2 > 0)
  for (int i = threadIdx.x; i < ROWS * H; i += MT) {
    const int r = i / H, j = i % H;
    float a = 0.f;
    for (int k = 0; k < K; ++k) a = fmaf(b.dy[r][k], sw[OFF_W3 + j * K + k], a);
    b.dz2[r][j] = b.z2[r][j] > 0.f ? a : 0.f;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < ROWS * H; i += MT) {
    const int r = i / H, j = i % H;
    float a = 0.f;
    for (int q = 0; q < H; ++q) a = fmaf(b.dz2[r][q], sw[OFF_W2 + j * H + q], a);
    b.dz1[r][j] = b.z1[r][j] > 0.f ? a : 0.f;
  }
  __syncthreads();
  // parameter gradients of this block's rows (fixed summation order)
  float *out = part + (int64_t)blockIdx.x * P;
  for (int p = threadIdx.x; p < P; p += MT) {
    float g = 0.f;
    if (p < OFF_B1) {
      const int f = p / H, j = p % H;
      for (int r = 0; r < ROWS; ++r) g = fmaf(b.x[r][f], b.dz1[r][j], g);
    } else if (p < OFF_W2) {
      const int j = p - OFF_B1;
      for (int r = 0; r < ROWS; ++r) g += b.dz1[r][j];
    } else if (p < OFF_B2) {
      const int q = (p - OFF_W2) / H, j = (p - OFF_W2) % H;
      for (int r = 0; r < ROWS; ++r) g = fmaf(fmaxf(b.z1[r][q], 0.f), b.dz2[r][j], g);
    } else if (p < OFF_W3) {
      const int j = p - OFF_B2;
      for (int r = 0; r < ROWS; ++r) g += b.dz2[r][j];
    } else if (p < OFF_B3) {
      const int q = (p - OFF_W3) / K, k = (p - OFF_W3) % K;
      for (int r = 0; r < ROWS; ++r) g = fmaf(fmaxf(b.z2[r][q], 0.f), b.dy[r][k], g);
    } else {
      const int k = p - OFF_B3;
      for (int r = 0; r < ROWS; ++r) g += b.dy[r][k];
    }
    out[p] = g;
  }
}

__global__ void mlp_reduce_kernel(const float *__restrict__ part, int nblk, const float *__restrict__ loss_part,
                                  float *__restrict__ grad, float *__restrict__ loss) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < P) {
    float g = 0.f;
    for (int i = 0; i < nblk; ++i) g += part[(int64_t)i * P + p];
    grad[p] = g;
  }
  if (p == 0) {
    float l = 0.f;
    for (int i = 0; i < nblk; ++i) l += loss_part[i];
    *loss = l;
  }
}

__global__ void mlp_adam_kernel(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m1,
                                float *__restrict__ m2, float lr, float wd, float bc1, float bc2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const float gp = g[p];
  const float a = 0.9f * m1[p] + 0.1f * gp;
  const float v = 0.999f * m2[p] + 0.001f * gp * gp;
  m1[p] = a;
  m2[p] = v;
  w[p] -= lr * ((a / bc1) / (sqrtf(v / bc2) + 1e-8f) + wd * w[p]);  // decoupled weight decay (AdamW)
}

// Inference for host-supplied rows, with the plan kernel's bf16 rounding.
__global__ void __launch_bounds__(MT) mlp_predict_kernel(const float *__restrict__ w, const float *__restrict__ X,
                                                        int64_t rows, float *__restrict__ out) {
  extern __shared__ float sw[];
  for (int i = threadIdx.x; i < P; i += MT) sw[i] = __bfloat162float(__float2bfloat16(w[i]));
  __syncthreads();
  const int64_t r = (int64_t)blockIdx.x * MT + threadIdx.x;
  if (r >= rows) return;
  float x[F], h1[H], h2[H];
  for (int f = 0; f < F; ++f) x[f] = X[r * F + f];
  for (int j = 0; j < H; ++j) {
    float a = sw[OFF_B1 + j];
    for (int f = 0; f < F; ++f) a = fmaf(x[f], sw[OFF_W1 + f * H + j], a);
    h1[j] = fmaxf(a, 0.f);
  }
  for (int j = 0; j < H; ++j) {
    float a = sw[OFF_B2 + j];
    for (int q = 0; q < H; ++q) a = fmaf(h1[q], sw[OFF_W2 + q * H + j], a);
    h2[j] = fmaxf(a, 0.f);
  }
  for (int k = 0; k < K; ++k) {
    float a = 0.f;
    for (int q = 0; q < H; ++q) a = fmaf(h2[q], sw[OFF_W3 + q * K + k], a);
    out[r * K + k] = a + sw[OFF_B3 + k];
  }
}

static size_t fwd_bwd_smem() { return sizeof(RowBuf) + P * sizeof(float); }

// Targets: log2(1 + cost) centred per row.
static void make_targets(const float *costs, int64_t rows, std::vector<float> &y) {
  y.resize((size_t)rows * K);
  for (int64_t r = 0; r < rows; ++r) {
    float mean = 0.f;
    for (int k = 0; k < K; ++k) {
      const float v = std::log2(1.0f + std::max(0.0f, costs[r * K + k]));
      y[(size_t)(r * K + k)] = v;
      mean += v;
    }
    mean /= (float)K;
    for (int k = 0; k < K; ++k) y[(size_t)(r * K + k)] -= mean;
  }
}

static void init_weights(uint64_t seed, std::vector<float> &w) {
  w.assign(P, 0.f);
  const uint64_t key = tc_stream_key(seed, 77);
  auto uni = [&](uint64_t i) { return (float)((tc_rand_at(key, i) >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f; };
  const float s1 = std::sqrt(6.f / F), s2 = std::sqrt(6.f / H), s3 = std::sqrt(3.f / H);
  for (int i = 0; i < F * H; ++i) w[OFF_W1 + i] = s1 * uni(i);
  for (int i = 0; i < H * H; ++i) w[OFF_W2 + i] = s2 * uni(100000 + i);
  for (int i = 0; i < H * K; ++i) w[OFF_W3 + i] = s3 * uni(200000 + i);
}

}  // namespace tc

extern "C" {

tc_status tc_selector_set_margin(tc_ctx *ctx, float margin) {
  if (!ctx || !(margin >= 0.f) || margin > 64.f)
    return set_error(ctx, TC_ERR_INVALID_ARG, "margin must lie in [0, 64]");
  ctx->mlp_margin = margin;
  return TC_OK;
}

tc_status tc_selector_set_weights(tc_ctx *ctx, const float *params, int64_t count) {
  if (!ctx || !params || count != P) return set_error(ctx, TC_ERR_INVALID_ARG, "expected %d parameters", P);
  TC_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(ctx->d_mlp, params, sizeof(float) * P, cudaMemcpyHostToDevice, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->mlp_loaded = true;
  return TC_OK;
}

tc_status tc_selector_get_weights(tc_ctx *ctx, float *params, int64_t count) {
  if (!ctx || !params || count != P) return set_error(ctx, TC_ERR_INVALID_ARG, "expected %d parameters", P);
  if (!ctx->mlp_loaded) return set_error(ctx, TC_ERR_INVALID_ARG, "no weights loaded");
  TC_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(params, ctx->d_mlp, sizeof(float) * P, cudaMemcpyDeviceToHost, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TC_OK;
}

tc_status tc_selector_predict(tc_ctx *ctx, const float *features, int64_t rows, float *pred) {
  if (!ctx || !features || !pred || rows < 0) return set_error(ctx, TC_ERR_INVALID_ARG, "bad argument");
  if (!ctx->mlp_loaded) return set_error(ctx, TC_ERR_INVALID_ARG, "no weights loaded");
  if (rows == 0) return TC_OK;
  TC_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  TC_TRY(arena_reserve(ctx, align_up(sizeof(float) * rows * F, 256) + align_up(sizeof(float) * rows * K, 256)));
  Bump bump{ctx->arena, ctx->arena_cap};
  float *dx = bump.take<float>(rows * F), *dy = bump.take<float>(rows * K);
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(dx, features, sizeof(float) * rows * F, cudaMemcpyHostToDevice, ctx->stream));
  mlp_predict_kernel<<<(int)((rows + MT - 1) / MT), MT, P * sizeof(float), ctx->stream>>>(ctx->d_mlp, dx, rows, dy);
  TC_CHECK_CUDA(ctx, cudaGetLastError());
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(pred, dy, sizeof(float) * rows * K, cudaMemcpyDeviceToHost, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TC_OK;
}

tc_status tc_selector_grad(tc_ctx *ctx, const float *params, const float *features, const float *targets,
                           int64_t rows, float *loss, float *grad) {
  if (!ctx || !params || !features || !targets || !loss || !grad || rows < 1)
    return set_error(ctx, TC_ERR_INVALID_ARG, "bad argument");
  TC_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  TC_CHECK_CUDA(ctx, cudaFuncSetAttribute(mlp_fwd_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)fwd_bwd_smem()));
  const int nblk = (int)((rows + ROWS - 1) / ROWS);
  Sizer sz;
  sz.take<float>(P); sz.take<float>(rows * F); sz.take<float>(rows * K);
  sz.take<float>((int64_t)nblk * P); sz.take<float>(nblk); sz.take<float>(P); sz.take<float>(1);
  TC_TRY(arena_reserve(ctx, sz.used));
  Bump bump{ctx->arena, ctx->arena_cap};
  float *dw = bump.take<float>(P), *dx = bump.take<float>(rows * F), *dt = bump.take<float>(rows * K);
  float *part = bump.take<float>((int64_t)nblk * P), *lp = bump.take<float>(nblk), *dg = bump.take<float>(P);
  float *dl = bump.take<float>(1);
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(dw, params, sizeof(float) * P, cudaMemcpyHostToDevice, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(dx, features, sizeof(float) * rows * F, cudaMemcpyHostToDevice, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(dt, targets, sizeof(float) * rows * K, cudaMemcpyHostToDevice, ctx->stream));
  const float inv = 1.0f / (float)(rows * K);
  mlp_fwd_bwd_kernel<<<nblk, MT, fwd_bwd_smem(), ctx->stream>>>(dw, dx, dt, nullptr, rows, inv, part, lp);
  TC_CHECK_CUDA(ctx, cudaGetLastError());
  mlp_reduce_kernel<<<(P + 255) / 256, 256, 0, ctx->stream>>>(part, nblk, lp, dg, dl);
  TC_CHECK_CUDA(ctx, cudaGetLastError());
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(grad, dg, sizeof(float) * P, cudaMemcpyDeviceToHost, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(loss, dl, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TC_OK;
}

tc_status tc_selector_train(tc_ctx *ctx, const float *features, const float *costs, int64_t rows, int32_t epochs,
                            float lr, float weight_decay, uint64_t seed, float *loss_out) {
  if (!ctx || !features || !costs || rows < 1 || epochs < 1 || !(lr > 0) || !(weight_decay >= 0))
    return set_error(ctx, TC_ERR_INVALID_ARG, "bad argument");
  TC_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  TC_CHECK_CUDA(ctx, cudaFuncSetAttribute(mlp_fwd_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)fwd_bwd_smem()));
  std::vector<float> y;
  make_targets(costs, rows, y);
  std::vector<float> w;
  init_weights(seed, w);
  const int64_t batch = std::min<int64_t>(rows, 1024);
  const int nblk = (int)((batch + ROWS - 1) / ROWS);
  Sizer sz;
  sz.take<float>(rows * F); sz.take<float>(rows * K); sz.take<int32_t>(rows);
  sz.take<float>((int64_t)nblk * P); sz.take<float>(nblk); sz.take<float>(P); sz.take<float>(P); sz.take<float>(P);
  sz.take<float>(1);
  TC_TRY(arena_reserve(ctx, sz.used));
  Bump bump{ctx->arena, ctx->arena_cap};
  float *dx = bump.take<float>(rows * F), *dt = bump.take<float>(rows * K);
  int32_t *didx = bump.take<int32_t>(rows);
  float *part = bump.take<float>((int64_t)nblk * P), *lp = bump.take<float>(nblk);
  float *dg = bump.take<float>(P), *m1 = bump.take<float>(P), *m2 = bump.take<float>(P), *dl = bump.take<float>(1);
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(dx, features, sizeof(float) * rows * F, cudaMemcpyHostToDevice, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(dt, y.data(), sizeof(float) * rows * K, cudaMemcpyHostToDevice, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(ctx->d_mlp, w.data(), sizeof(float) * P, cudaMemcpyHostToDevice, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(m1, 0, sizeof(float) * P, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(m2, 0, sizeof(float) * P, ctx->stream));
  std::vector<int32_t> perm((size_t)rows);
  for (int64_t i = 0; i < rows; ++i) perm[(size_t)i] = (int32_t)i;
  const uint64_t key = tc_stream_key(seed, 99);
  int64_t step = 0;
  float last = 0.f;
  for (int ep = 0; ep < epochs; ++ep) {
    for (int64_t i = rows - 1; i > 0; --i) {  // Fisher-Yates with the counter RNG
      const int64_t j = (int64_t)tc_mulhi(tc_rand_at(key, (uint64_t)(ep * rows + i)), (uint64_t)(i + 1));
      std::swap(perm[(size_t)i], perm[(size_t)j]);
    }
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(didx, perm.data(), sizeof(int32_t) * rows, cudaMemcpyHostToDevice, ctx->stream));
    TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // perm is pageable and rewritten next epoch
    for (int64_t b0 = 0; b0 < rows; b0 += batch) {
      const int64_t nb = std::min(batch, rows - b0);
      const int blk = (int)((nb + ROWS - 1) / ROWS);
      const float inv = 1.0f / (float)(nb * K);
      mlp_fwd_bwd_kernel<<<blk, MT, fwd_bwd_smem(), ctx->stream>>>(ctx->d_mlp, dx, dt, didx + b0, nb, inv, part, lp);
      mlp_reduce_kernel<<<(P + 255) / 256, 256, 0, ctx->stream>>>(part, blk, lp, dg, dl);
      ++step;
      const float bc1 = 1.f - std::pow(0.9f, (float)step), bc2 = 1.f - std::pow(0.999f, (float)step);
      mlp_adam_kernel<<<(P + 255) / 256, 256, 0, ctx->stream>>>(ctx->d_mlp, dg, m1, m2, lr, weight_decay, bc1, bc2);
    }
    TC_CHECK_CUDA(ctx, cudaGetLastError());
  }
  // final loss over every row (mean over rows and arms)
  for (int64_t b0 = 0; b0 < rows; b0 += batch) {
    const int64_t nb = std::min(batch, rows - b0);
    const int blk = (int)((nb + ROWS - 1) / ROWS);
    for (int64_t i = 0; i < nb; ++i) perm[(size_t)i] = (int32_t)(b0 + i);
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(didx, perm.data(), sizeof(int32_t) * nb, cudaMemcpyHostToDevice, ctx->stream));
    mlp_fwd_bwd_kernel<<<blk, MT, fwd_bwd_smem(), ctx->stream>>>(ctx->d_mlp, dx, dt, didx, nb,
                                                                 1.0f / (float)(rows * K), part, lp);
    mlp_reduce_kernel<<<(P + 255) / 256, 256, 0, ctx->stream>>>(part, blk, lp, dg, dl);
    float l = 0;
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&l, dl, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    last += l;
  }
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->mlp_loaded = true;
  if (loss_out) *loss_out = last;
  return TC_OK;
}

}  // extern "C"
