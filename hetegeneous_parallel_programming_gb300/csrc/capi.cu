// extern "C" entry points of libtc: ctx lifetime, orientation, counting,
// device generators and the device symmetric-CSR builder.
#include <algorithm>
#include <vector>

#include "engine.cuh"
#include "tc_gen_common.h"

using namespace tc;

namespace tc {

const char *flag_text(unsigned f) {
  if (f & VF_ROWPTR_ENDS) return "rowptr[0] must be 0 and rowptr[n] must equal nnz";
  if (f & VF_ROWPTR_ORDER) return "rowptr is not monotone";
  if (f & VF_ID_RANGE) return "a column id is outside [0, n)";
  if (f & VF_SELF_LOOP) return "a row holds a self loop";
  if (f & VF_UNSORTED) return "a row is not strictly ascending (unsorted or duplicate neighbours)";
  if (f & VF_TIMEOUT) return "a bounded device wait gave up";
  if (f & VF_PART_RANGE) return "a partition id is outside [0, num_parts)";
  return "invalid graph";
}

static tc_status check_csr_args(tc_ctx *ctx, const tc_csr *g) {
  if (!g) return set_error(ctx, TC_ERR_INVALID_ARG, "null graph");
  if (g->n < 1 || g->n > 2147483647LL)
    return set_error(ctx, TC_ERR_UNSUPPORTED, "n=%lld outside [1, 2^31-1]", (long long)g->n);
  if (g->nnz < 0 || !g->rowptr || (g->nnz > 0 && !g->colidx))
    return set_error(ctx, TC_ERR_INVALID_ARG, "bad nnz or null CSR arrays");
  if (g->nnz >= (int64_t(1) << 32))
    return set_error(ctx, TC_ERR_UNSUPPORTED, "nnz=%lld: this engine indexes oriented edges with 32 bits",
                     (long long)g->nnz);
  return TC_OK;
}

// Host-to-device copies of page-locked caller memory by the SMs: the
// kernel reads the host buffer through its mapping over the C2C link.  On the
// GB300 machines measured, the copy engines' rate fell from 211 GB/s to 100-157
// GB/s for some copies after seconds of device load, while this kernel held
// 211 GB/s throughout.  dst is 16-byte aligned (arena); src is whatever the
// caller passed: a 16-byte body when both share their offset mod 16, else
// 4-byte words (the CSR's element size), with the bytes' count a multiple of 4.
__global__ void h2d_copy_kernel(const char *__restrict__ src, char *__restrict__ dst, size_t bytes) {
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x, nt = (size_t)gridDim.x * blockDim.x;
  const size_t head = (16 - (reinterpret_cast<uintptr_t>(dst) & 15)) & 15;
  if (((reinterpret_cast<uintptr_t>(src) ^ reinterpret_cast<uintptr_t>(dst)) & 15) == 0 && bytes >= head) {
    for (size_t i = tid; i < head / 4; i += nt)
      reinterpret_cast<uint32_t *>(dst)[i] = reinterpret_cast<const uint32_t *>(src)[i];
    const size_t n16 = (bytes - head) / 16;
    const uint4 *s16 = reinterpret_cast<const uint4 *>(src + head);
    uint4 *d16 = reinterpret_cast<uint4 *>(dst + head);
    for (size_t i = tid; i < n16; i += nt) d16[i] = s16[i];
    const size_t done = head + 16 * n16;
    for (size_t i = tid; i < (bytes - done) / 4; i += nt)
      reinterpret_cast<uint32_t *>(dst + done)[i] = reinterpret_cast<const uint32_t *>(src + done)[i];
  } else {
    for (size_t i = tid; i < bytes / 4; i += nt)
      reinterpret_cast<uint32_t *>(dst)[i] = reinterpret_cast<const uint32_t *>(src)[i];
  }
}

// The device address of page-locked host memory, or null (pageable memory,
// or TC_H2D_KERNEL 0): the caller then copies with cudaMemcpyAsync.
#ifndef TC_H2D_KERNEL
#define TC_H2D_KERNEL 1
#endif
#ifndef TC_H2D_BLOCKS_PER_SM
#define TC_H2D_BLOCKS_PER_SM 1  // R-MAT scale 24 e2e: 1 60.76 ms, 2 61.31, 4 62.59 (the copy shares the SMs)
#endif
static const void *mapped_host(const void *p) {
  if (!TC_H2D_KERNEL || !p) return nullptr;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

static tc_status h2d_copy(tc_ctx *ctx, void *dst, const void *src, const void *src_dev, size_t bytes,
                          cudaStream_t st) {
  if (bytes == 0) return TC_OK;
  if (src_dev) {
    h2d_copy_kernel<<<ctx->num_sms * TC_H2D_BLOCKS_PER_SM, 256, 0, st>>>(static_cast<const char *>(src_dev),
                                                     static_cast<char *>(dst), bytes);
    TC_CHECK_LAUNCH(ctx);
  } else {
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
  }
  return TC_OK;
}

// Device copies of a caller CSR (no copy when already on the device).
tc_status stage_csr(tc_ctx *ctx, const tc_csr *g, Bump &bump, DevCSR &d, uint64_t *h2d, int pieces) {
  d.n = g->n;
  d.nnz = g->nnz;
  if (g->on_device) {
    d.rowptr = g->rowptr;
    d.col = g->colidx;
    return TC_OK;
  }
  int64_t *rp = bump.take<int64_t>(g->n + 1);
  int32_t *cl = bump.take<int32_t>(g->nnz);
  if (bump.overflow) return set_error(ctx, TC_ERR_OOM, "arena overflow staging the graph");
  const void *rp_dev = mapped_host(g->rowptr);
  const char *cl_dev = static_cast<const char *>(g->nnz > 0 ? mapped_host(g->colidx) : nullptr);
  TC_TRY(h2d_copy(ctx, rp, g->rowptr, rp_dev, sizeof(int64_t) * (size_t)(g->n + 1), ctx->stream));
  if (pieces > 1) {
    // piece k = blocks [k * per, (k + 1) * per) of the kept-count geometry
    int G;
    int64_t chunk;
    orient_geometry(ctx, g->nnz, pieces, &G, &chunk);
    const int per = (G + pieces - 1) / pieces;
    TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->piece_ev[0], ctx->stream));
    TC_CHECK_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->piece_ev[0], 0));
    for (int k = 0; k < pieces; ++k) {
      const int64_t e0 = std::min<int64_t>(g->nnz, (int64_t)k * per * chunk);
      const int64_t e1 = std::min<int64_t>(g->nnz, (int64_t)(k + 1) * per * chunk);
      if (e1 > e0)
        TC_TRY(h2d_copy(ctx, cl + e0, g->colidx + e0, cl_dev ? cl_dev + sizeof(int32_t) * (size_t)e0 : nullptr,
                        sizeof(int32_t) * (size_t)(e1 - e0), ctx->copy_stream));
      TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->piece_ev[k], ctx->copy_stream));
    }
  } else if (g->nnz > 0) {
    TC_TRY(h2d_copy(ctx, cl, g->colidx, cl_dev, sizeof(int32_t) * (size_t)g->nnz, ctx->stream));
  }
  *h2d += sizeof(int64_t) * (size_t)(g->n + 1) + sizeof(int32_t) * (size_t)g->nnz;
  d.rowptr = rp;
  d.col = cl;
  return TC_OK;
}

void orient_sizes(const tc_ctx *ctx, int64_t n, int64_t nnz, bool perm, bool dagcol, Sizer &sz, int pieces) {
  int G;
  int64_t chunk;
  orient_geometry(ctx, nnz, pieces, &G, &chunk);
  const int64_t mmax = nnz;
  sz.take<uint64_t>(n); sz.take<uint64_t>(n);
  sz.take<int32_t>(n);
  sz.take<int64_t>(n + 1);
  sz.take<int64_t>(G + 1);
  sz.take<int64_t>(1);
  size_t scr = std::max(radix_sort_scratch_bytes(ctx, std::max<int64_t>(n, mmax)), scan_scratch_bytes(ctx, n + 1));
  scr = std::max(scr, scan_scratch_bytes(ctx, G));
  sz.take<char>((int64_t)scr);
  sz.take<int64_t>(n + 1); sz.take<int64_t>(n + 1); sz.take<int64_t>(n + 1);
  sz.take<int2>(n);
  sz.take<int32_t>(n); sz.take<int32_t>(n); sz.take<int32_t>(n); sz.take<unsigned>(4);
  sz.take<int32_t>(nnz);
  sz.take<int32_t>(mmax); sz.take<int32_t>(mmax);
  if (perm) sz.take<uint32_t>(mmax);
  if (dagcol) sz.take<int32_t>(mmax);
}

void orient_carve(const tc_ctx *ctx, int64_t n, int64_t nnz, bool perm, bool dagcol, Bump &bump,
                         OrientBufs &b, int pieces) {
  b.pieces = pieces;
  orient_geometry(ctx, nnz, pieces, &b.G, &b.chunk);
  const int64_t mmax = nnz;
  b.vkeys0 = bump.take<uint64_t>(n);
  b.vkeys1 = bump.take<uint64_t>(n);
  b.rank = bump.take<int32_t>(n);
  b.kept = bump.take<int64_t>(n + 1);
  b.bcount = bump.take<int64_t>(b.G + 1);
  b.d_m = bump.take<int64_t>(1);
  size_t scr = std::max(radix_sort_scratch_bytes(ctx, std::max<int64_t>(n, mmax)), scan_scratch_bytes(ctx, n + 1));
  scr = std::max(scr, scan_scratch_bytes(ctx, b.G));
  b.sort_scratch = bump.take<char>((int64_t)scr);
  b.orowptr = bump.take<int64_t>(n + 1);
  b.nrowptr = bump.take<int64_t>(n + 1);
  b.dnew = bump.take<int64_t>(n + 1);
  b.dv = bump.take<int2>(n);
  b.mid_list = bump.take<int32_t>(n);
  b.big_list = bump.take<int32_t>(n);
  b.huge_list = bump.take<int32_t>(n);
  b.seg_counts = bump.take<unsigned>(4);
  b.rv = bump.take<int32_t>(nnz);
  b.ncol = bump.take<int32_t>(mmax);
  b.nsrc = bump.take<int32_t>(mmax);
  b.perm = perm ? bump.take<uint32_t>(mmax) : nullptr;
  b.dag_col = dagcol ? bump.take<int32_t>(mmax) : nullptr;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return ms;
}

// Validation + phase A + read back m and the flags (which the caller zeroed
// before any kernel that may set them).
// The orientation's first half up to the host's read of m and the flags
// (the copies are queued, not waited for); graph-capturable.
tc_status orient_front_launch(tc_ctx *ctx, const DevCSR &d, const tc_opts &o, OrientBufs &ob) {
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[1], ctx->stream));
  // row pointers here; the column checks ride on the kept-count pass
  if (o.validate) TC_TRY(launch_validate_rowptr(ctx, d));
  ob.validate = o.validate != 0;
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[2], ctx->stream));
  TC_TRY(orient_phase_a(ctx, d, ob));
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[3], ctx->stream));
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ctx->h_pinned[0], ob.d_m, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ctx->h_pinned[1], ctx->d_flags, sizeof(unsigned) * 2, cudaMemcpyDeviceToHost,
                                     ctx->stream));
  return TC_OK;
}

// Waits for orient_front_launch's copies: the validation flags and m.
tc_status orient_front_finish(tc_ctx *ctx, int64_t *m, float *ms_validate, float *ms_a) {
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const unsigned flags = (unsigned)(ctx->h_pinned[1] & 0xffffffffu);
  if (flags) return set_error(ctx, TC_ERR_INVALID_GRAPH, "%s", flag_text(flags));
  *m = (int64_t)ctx->h_pinned[0];
  *ms_validate = elapsed(ctx->ev[1], ctx->ev[2]);
  *ms_a = elapsed(ctx->ev[2], ctx->ev[3]);
  return TC_OK;
}

tc_status orient_front(tc_ctx *ctx, const DevCSR &d, const tc_opts &o, OrientBufs &ob, int64_t *m,
                              float *ms_validate, float *ms_a) {
  TC_TRY(orient_front_launch(ctx, d, o, ob));
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const unsigned flags = (unsigned)(ctx->h_pinned[1] & 0xffffffffu);
  if (flags) return set_error(ctx, TC_ERR_INVALID_GRAPH, "%s", flag_text(flags));
  *m = (int64_t)ctx->h_pinned[0];
  *ms_validate = elapsed(ctx->ev[1], ctx->ev[2]);
  *ms_a = elapsed(ctx->ev[2], ctx->ev[3]);
  return TC_OK;
}

// L2 read probe: every thread strides the buffer with 16-byte L2-only loads,
// `passes` times; the XOR of what it read keeps the loads alive.
__global__ void l2_read_kernel(const uint4 *__restrict__ buf, int64_t n4, int passes, unsigned *sink) {
  uint32_t acc = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int p = 0; p < passes; ++p) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n4; i += 4 * stride) {
      const uint4 a = __ldcg(buf + i), b = __ldcg(buf + i + stride), c = __ldcg(buf + i + 2 * stride),
                  d = __ldcg(buf + i + 3 * stride);
      acc ^= a.x ^ a.y ^ a.z ^ a.w ^ b.x ^ b.y ^ b.z ^ b.w ^ c.x ^ c.y ^ c.z ^ c.w ^ d.x ^ d.y ^ d.z ^ d.w;
    }
    for (; i < n4; i += stride) {
      const uint4 a = __ldcg(buf + i);
      acc ^= a.x ^ a.y ^ a.z ^ a.w;
    }
  }
  if (acc == 0x9e3779b9u) atomicAdd(sink, 1u);  // practically never taken
}

}  // namespace tc

// A bounded device-side wait that gave up (VF_TIMEOUT, read back with the
// total into h_pinned[3]) fails the call.  The kernels that wait count the
// affected edges without the staged copy, so the total is still exact, but
// a wait that runs out points at a device that is not making progress.
static tc_status check_wait_flags(tc_ctx *ctx) {
  if ((unsigned)(ctx->h_pinned[3] & 0xffffffffu) & VF_TIMEOUT)
    return set_error(ctx, TC_ERR_TIMEOUT, "a bounded device wait gave up (bulk copy not completed)");
  return TC_OK;
}

extern "C" {

tc_status tc_set_pull_chunks(tc_ctx *ctx, int32_t item, int32_t item_min) {
  if (!ctx) return set_error(ctx, TC_ERR_INVALID_ARG, "null ctx");
  if (item_min < 32 || item_min > item || item > 65536)
    return set_error(ctx, TC_ERR_INVALID_ARG, "need 32 <= item_min <= item <= 65536 (got %d, %d)", (int)item_min,
                     (int)item);
  ctx->pull_item = item;
  ctx->pull_item_min = item_min;
  return TC_OK;
}

tc_status tc_get_pull_chunks(const tc_ctx *ctx, int32_t *item, int32_t *item_min) {
  if (!ctx || !item || !item_min) return set_error(nullptr, TC_ERR_INVALID_ARG, "null argument");
  *item = ctx->pull_item;
  *item_min = ctx->pull_item_min;
  return TC_OK;
}

tc_status tc_autotune_pull(tc_ctx *ctx, const tc_csr *g, const tc_opts *opts, const int32_t *candidates,
                           int32_t ncand, int32_t reps, float *ms, int32_t *best) {
  if (!ctx || !candidates || ncand < 1 || reps < 1)
    return set_error(ctx, TC_ERR_INVALID_ARG, "need ctx, candidates, ncand >= 1 and reps >= 1");
  for (int32_t i = 0; i < ncand; ++i)
    if (candidates[i] < 32 || candidates[i] > 65536)
      return set_error(ctx, TC_ERR_INVALID_ARG, "candidate %d outside [32, 65536]", (int)candidates[i]);
  const int old_item = ctx->pull_item, old_min = ctx->pull_item_min;
  auto restore = [&](tc_status st) {
    ctx->pull_item = old_item;
    ctx->pull_item_min = old_min;
    return st;
  };
  float best_ms = 0.f;
  int32_t best_item = old_item;
  uint64_t first_total = 0;
  for (int32_t i = 0; i < ncand; ++i) {
    ctx->pull_item = candidates[i];
    ctx->pull_item_min = std::max(32, candidates[i] / 4);
    float cand_ms = 0.f;
    for (int32_t r = 0; r <= reps; ++r) {  // r == 0 warms up
      uint64_t total = 0;
      tc_stats st;
      const tc_status s = tc_count(ctx, g, opts, &total, nullptr, 0, &st);
      if (s != TC_OK) return restore(s);
      if (i == 0 && r == 0) first_total = total;
      if (total != first_total)
        return restore(set_error(ctx, TC_ERR_INVALID_GRAPH,
                                 "chunk size %d counted %llu triangles, %llu with the first candidate",
                                 (int)candidates[i], (unsigned long long)total, (unsigned long long)first_total));
      if (r > 0 && (cand_ms == 0.f || st.ms_total < cand_ms)) cand_ms = st.ms_total;
    }
    if (ms) ms[i] = cand_ms;
    if (i == 0 || cand_ms < best_ms) {
      best_ms = cand_ms;
      best_item = candidates[i];
    }
  }
  ctx->pull_item = best_item;
  ctx->pull_item_min = std::max(32, best_item / 4);
  if (best) *best = best_item;
  return TC_OK;
}

tc_status tc_get_tuning(const tc_ctx *ctx, tc_tuning *out) {
  if (!ctx || !out) return set_error(nullptr, TC_ERR_INVALID_ARG, "null ctx or tuning");
  out->pull_item = ctx->pull_item;
  out->pull_item_min = ctx->pull_item_min;
  out->pull_block_tiles = ctx->pull_block_tiles;
  out->pull_dense_num = ctx->pull_dense_num;
  out->pull_dense_den = ctx->pull_dense_den;
  out->orient_blocks_per_sm = ctx->orient_blocks_per_sm;
  return TC_OK;
}

tc_status tc_set_tuning(tc_ctx *ctx, const tc_tuning *t) {
  if (!ctx || !t) return set_error(ctx, TC_ERR_INVALID_ARG, "null ctx or tuning");
  if (t->pull_item_min < 32 || t->pull_item < t->pull_item_min || t->pull_item > 65536)
    return set_error(ctx, TC_ERR_INVALID_ARG, "PULL chunks need 32 <= item_min <= item <= 65536");
  if (t->pull_block_tiles < 64 || t->pull_block_tiles > (1 << 20))
    return set_error(ctx, TC_ERR_INVALID_ARG, "pull_block_tiles %d outside [64, 2^20]", (int)t->pull_block_tiles);
  if (t->pull_dense_num < 1 || t->pull_dense_num > 64 || t->pull_dense_den < 1 || t->pull_dense_den > 64)
    return set_error(ctx, TC_ERR_INVALID_ARG, "dense ratio terms outside [1, 64]");
  if (t->orient_blocks_per_sm < 1 || t->orient_blocks_per_sm > 64)
    return set_error(ctx, TC_ERR_INVALID_ARG, "orient_blocks_per_sm %d outside [1, 64]", (int)t->orient_blocks_per_sm);
  ctx->pull_item = t->pull_item;
  ctx->pull_item_min = t->pull_item_min;
  ctx->pull_block_tiles = t->pull_block_tiles;
  ctx->pull_dense_num = t->pull_dense_num;
  ctx->pull_dense_den = t->pull_dense_den;
  ctx->orient_blocks_per_sm = t->orient_blocks_per_sm;
  return TC_OK;
}

tc_status tc_autotune(tc_ctx *ctx, const tc_csr *g, const tc_opts *opts, int32_t reps, tc_tuning *best,
                      float *best_ms, int32_t *trials) {
  if (!ctx || !g || reps < 1) return set_error(ctx, TC_ERR_INVALID_ARG, "need ctx, graph and reps >= 1");
  tc_tuning old, cur;
  TC_TRY(tc_get_tuning(ctx, &old));
  cur = old;
  uint64_t first_total = 0;
  bool have_total = false;
  int32_t ntrials = 0;
  // time one setting: a warm-up call, then the best of `reps` calls
  auto trial = [&](const tc_tuning &t, float *ms_out) -> tc_status {
    TC_TRY(tc_set_tuning(ctx, &t));
    float best_t = 0.f;
    for (int32_t r = 0; r <= reps; ++r) {
      uint64_t total = 0;
      tc_stats st;
      TC_TRY(tc_count(ctx, g, opts, &total, nullptr, 0, &st));
      if (!have_total) {
        first_total = total;
        have_total = true;
      }
      if (total != first_total)
        return set_error(ctx, TC_ERR_INVALID_GRAPH, "a tuning trial counted %llu triangles, the first %llu",
                         (unsigned long long)total, (unsigned long long)first_total);
      if (r > 0 && (best_t == 0.f || st.ms_total < best_t)) best_t = st.ms_total;
    }
    ++ntrials;
    *ms_out = best_t;
    return TC_OK;
  };
  float cur_ms = 0.f;
  tc_status s = trial(cur, &cur_ms);
  for (int dim = 0; s == TC_OK && dim < 4; ++dim) {
    for (int c = 0; s == TC_OK && c < 3; ++c) {
      tc_tuning t = cur;
      if (dim == 0) {
        static const int items[3] = {256, 512, 1024};
        t.pull_item = items[c];
        t.pull_item_min = std::max(32, items[c] / 4);
      } else if (dim == 1) {
        static const int tiles[3] = {1280, 2560, 5120};
        t.pull_block_tiles = tiles[c];
      } else if (dim == 2) {
        static const int num[3] = {1, 1, 2}, den[3] = {2, 1, 1};
        t.pull_dense_num = num[c];
        t.pull_dense_den = den[c];
      } else {
        static const int bps[3] = {3, 6, 12};
        t.orient_blocks_per_sm = bps[c];
      }
      if (memcmp(&t, &cur, sizeof(t)) == 0) continue;  // already timed
      float ms = 0.f;
      s = trial(t, &ms);
      if (s == TC_OK && ms < cur_ms) {
        cur = t;
        cur_ms = ms;
      }
    }
  }
  if (s != TC_OK) {
    (void)tc_set_tuning(ctx, &old);
    return s;
  }
  TC_TRY(tc_set_tuning(ctx, &cur));
  if (best) *best = cur;
  if (best_ms) *best_ms = cur_ms;
  if (trials) *trials = ntrials;
  return TC_OK;
}

tc_status tc_l2_bandwidth(tc_ctx *ctx, int64_t bytes, int32_t passes, double *gbs) {
  if (!ctx || !gbs || bytes < 4096 || passes < 1)
    return set_error(ctx, TC_ERR_INVALID_ARG, "need ctx, gbs, bytes >= 4096 and passes >= 1");
  TC_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  const int64_t n4 = bytes / 16;
  TC_TRY(arena_reserve(ctx, n4 * 16 + 256));
  uint4 *buf = reinterpret_cast<uint4 *>(ctx->arena);
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(buf, 1, (size_t)n4 * 16, ctx->stream));
  const int grid = ctx->num_sms * 8;
  float best = 0.f;
  for (int rep = 0; rep < 6; ++rep) {
    TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
    l2_read_kernel<<<grid, 256, 0, ctx->stream>>>(buf, n4, passes, ctx->d_flags + 7);
    TC_CHECK_LAUNCH(ctx);
    TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[1], ctx->stream));
    TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const float ms = elapsed(ctx->ev[0], ctx->ev[1]);
    if (rep > 0 && (best == 0.f || ms < best)) best = ms;  // rep 0 warms up
  }
  *gbs = best > 0.f ? (double)n4 * 16.0 * passes / (best * 1e-3) / 1e9 : 0.0;
  return TC_OK;
}

tc_status tc_ctx_create(int device, tc_ctx **out) {
  if (!out) return set_error(nullptr, TC_ERR_INVALID_ARG, "null out");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    (void)cudaGetLastError();
    return set_error(nullptr, TC_ERR_NO_DEVICE, "no CUDA device (%s)", cudaGetErrorString(e));
  }
  if (device < 0 || device >= count)
    return set_error(nullptr, TC_ERR_INVALID_ARG, "device %d outside [0,%d)", device, count);
  tc_ctx *ctx = new tc_ctx();
  ctx->device = device;
  auto fail = [&](tc_status st) {
    tc_ctx_destroy(ctx);
    return st;
  };
  if (cudaSetDevice(device) != cudaSuccess) return fail(set_error(nullptr, TC_ERR_CUDA, "cudaSetDevice failed"));
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess)
    return fail(set_error(nullptr, TC_ERR_CUDA, "cudaGetDeviceProperties failed"));
  ctx->num_sms = prop.multiProcessorCount;
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(set_error(nullptr, TC_ERR_CUDA, "stream creation failed"));
  for (auto &ev : ctx->ev)
    if (cudaEventCreate(&ev) != cudaSuccess) return fail(set_error(nullptr, TC_ERR_CUDA, "event creation failed"));
  for (auto &ev : ctx->piece_ev)
    if (cudaEventCreate(&ev) != cudaSuccess) return fail(set_error(nullptr, TC_ERR_CUDA, "event creation failed"));
  if (cudaMalloc((void **)&ctx->d_total, 256) != cudaSuccess || cudaMalloc((void **)&ctx->d_flags, 256) != cudaSuccess ||
      cudaMalloc((void **)&ctx->d_heads, 256) != cudaSuccess ||
      cudaMalloc((void **)&ctx->d_mlp, TC_MLP_PARAM_COUNT * sizeof(float)) != cudaSuccess ||
      cudaMallocHost((void **)&ctx->h_pinned, 64 * sizeof(unsigned long long)) != cudaSuccess) {
    (void)cudaGetLastError();
    return fail(set_error(nullptr, TC_ERR_OOM, "ctx state allocation failed"));
  }
  tc_status st = init_arm_occupancy(ctx);
  if (st != TC_OK) return fail(st);
  *out = ctx;
  return TC_OK;
}

void tc_ctx_destroy(tc_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);  // pieced uploads write the arena
  cudaFree(ctx->arena);
  cudaFree(ctx->aux);
  cudaFree(ctx->d_total);
  cudaFree(ctx->d_flags);
  cudaFree(ctx->d_heads);
  cudaFree(ctx->d_mlp);
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  if (ctx->batch_exec) cudaGraphExecDestroy(ctx->batch_exec);
  if (ctx->batch_front_exec) cudaGraphExecDestroy(ctx->batch_front_exec);
  for (auto &ev : ctx->ev)
    if (ev) cudaEventDestroy(ev);
  for (auto &ev : ctx->piece_ev)
    if (ev) cudaEventDestroy(ev);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  (void)cudaGetLastError();
  delete ctx;
}

const char *tc_last_error(const tc_ctx *ctx) { return ctx ? ctx->err : global_error(); }

int64_t tc_ctx_arena_bytes(const tc_ctx *ctx) { return ctx ? (int64_t)ctx->arena_cap : 0; }

void *tc_ctx_stream(tc_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

tc_status tc_ctx_sync(tc_ctx *ctx) {
  if (!ctx) return set_error(nullptr, TC_ERR_INVALID_ARG, "null ctx");
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TC_OK;
}

tc_status tc_count(tc_ctx *ctx, const tc_csr *g, const tc_opts *opts_in, uint64_t *total, uint32_t *edge_counts,
                   int64_t edge_capacity, tc_stats *stats) {
  if (!ctx || !total) return set_error(ctx, TC_ERR_INVALID_ARG, "null ctx or total");
  TC_TRY(check_csr_args(ctx, g));
  tc_opts o;
  tc_opts_default(&o);
  if (opts_in) o = *opts_in;
  TC_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  ctx->launches = 0;
  tc_stats st;
  memset(&st, 0, sizeof(st));
  const bool want_edges = edge_counts != nullptr;
  // host input: the column array uploads in pieces behind the orientation's
  // first passes (worth it once the upload takes milliseconds)
  const int pieces = (!g->on_device && g->nnz >= (int64_t(1) << 24)) ? TC_MAX_PIECES : 1;
  // arena: staged input + orientation + counting + output staging
  Sizer sz;
  if (!g->on_device) { sz.take<int64_t>(g->n + 1); sz.take<int32_t>(g->nnz); }
  orient_sizes(ctx, g->n, g->nnz, want_edges, false, sz, pieces);
  sz.used += count_scratch_bytes(ctx, g->n, g->nnz);
  if (want_edges && !g->on_device) sz.take<uint32_t>(g->nnz);
  TC_TRY(arena_reserve(ctx, sz.used));
  Bump bump{ctx->arena, ctx->arena_cap};
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned) * 8, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
  // every return waits for the pieces' uploads: none may outlive the call
  // (the arena and the caller's host arrays are only borrowed)
  struct UploadGuard {
    tc_ctx *c;
    bool on;
    ~UploadGuard() {
      if (on) cudaStreamSynchronize(c->copy_stream);
    }
  } upload_guard{ctx, pieces > 1};
  DevCSR d;
  TC_TRY(stage_csr(ctx, g, bump, d, &st.h2d_bytes, pieces));
  OrientBufs ob;
  orient_carve(ctx, d.n, d.nnz, want_edges, false, bump, ob, pieces);
  CountBufs cb;
  if (count_carve(ctx, d.n, d.nnz, bump, cb, o.record_tile_costs != 0) != TC_OK || bump.overflow)
    return set_error(ctx, TC_ERR_OOM, "arena overflow");
  uint32_t *d_out = nullptr;
  if (want_edges) d_out = g->on_device ? edge_counts : bump.take<uint32_t>(d.nnz);
  int64_t m = 0;
  float ms_a = 0;
  TC_TRY(orient_front(ctx, d, o, ob, &m, &st.ms_validate, &ms_a));
  // with pieces the upload ends at the last piece's event (it overlaps the orientation)
  st.ms_h2d = elapsed(ctx->ev[0], pieces > 1 ? ctx->piece_ev[pieces - 1] : ctx->ev[1]);
  if (want_edges && edge_capacity < m)
    return set_error(ctx, TC_ERR_INVALID_ARG, "edge_counts holds %lld entries, %lld oriented edges",
                     (long long)edge_capacity, (long long)m);
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[4], ctx->stream));
  DevDag dag;
  TC_TRY(orient_phase_b(ctx, d, ob, m, want_edges, false, &dag));
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[5], ctx->stream));
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_total, 0, sizeof(unsigned long long), ctx->stream));
  TC_TRY(run_count(ctx, dag, o, cb, d_out, true));
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[6], ctx->stream));
  if (want_edges && !g->on_device && m > 0) {
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(edge_counts, d_out, sizeof(uint32_t) * (size_t)m, cudaMemcpyDeviceToHost,
                                       ctx->stream));
    st.d2h_bytes += sizeof(uint32_t) * (size_t)m;
  }
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ctx->h_pinned[2], ctx->d_total, sizeof(unsigned long long),
                                     cudaMemcpyDeviceToHost, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ctx->h_pinned[3], ctx->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost,
                                     ctx->stream));
  st.d2h_bytes += sizeof(unsigned long long);
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[7], ctx->stream));
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  TC_TRY(check_wait_flags(ctx));
  *total = ctx->h_pinned[2];
  count_stats(ctx, &st, true);
  st.ms_orient = ms_a + elapsed(ctx->ev[4], ctx->ev[5]);
  st.ms_d2h = elapsed(ctx->ev[6], ctx->ev[7]);
  st.ms_total = elapsed(ctx->ev[0], ctx->ev[7]);
  st.m = m;
  st.tiles = (m + TILE_EDGES - 1) / TILE_EDGES;
  st.kernel_launches = ctx->launches;
  if (stats) *stats = st;
  return TC_OK;
}


// Labelled counts: for every oriented edge u->v, the common out-neighbours w
// whose label is `label` (the reference's labelled intersection, on the DAG).
tc_status tc_count_labelled(tc_ctx *ctx, const tc_csr *g, const uint8_t *vertex_labels, int32_t label,
                            const tc_opts *opts_in, uint64_t *total, uint32_t *edge_counts, int64_t edge_capacity,
                            tc_stats *stats) {
  if (!ctx || !total || !vertex_labels) return set_error(ctx, TC_ERR_INVALID_ARG, "null ctx, total or vertex_labels");
  if (label < 0 || label > 255) return set_error(ctx, TC_ERR_INVALID_ARG, "label %d outside [0, 255]", label);
  TC_TRY(check_csr_args(ctx, g));
  tc_opts o;
  tc_opts_default(&o);
  if (opts_in) o = *opts_in;
  o.selector = TC_SELECT_FORCE;  // only the PULL arm filters hits by label
  o.force_arm = TC_ARM_PULL;
  TC_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  ctx->launches = 0;
  tc_stats st;
  memset(&st, 0, sizeof(st));
  const bool want_edges = edge_counts != nullptr;
  Sizer sz;
  if (!g->on_device) { sz.take<int64_t>(g->n + 1); sz.take<int32_t>(g->nnz); sz.take<uint8_t>(g->n); }
  orient_sizes(ctx, g->n, g->nnz, want_edges, false, sz);
  sz.used += count_scratch_bytes(ctx, g->n, g->nnz);
  sz.take<uint8_t>(g->n);
  if (want_edges && !g->on_device) sz.take<uint32_t>(g->nnz);
  TC_TRY(arena_reserve(ctx, sz.used));
  Bump bump{ctx->arena, ctx->arena_cap};
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned) * 8, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
  DevCSR d;
  TC_TRY(stage_csr(ctx, g, bump, d, &st.h2d_bytes));
  const uint8_t *d_lab_in = vertex_labels;
  if (!g->on_device) {
    uint8_t *tmp = bump.take<uint8_t>(d.n);
    if (bump.overflow) return set_error(ctx, TC_ERR_OOM, "arena overflow");
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(tmp, vertex_labels, (size_t)d.n, cudaMemcpyHostToDevice, ctx->stream));
    st.h2d_bytes += (uint64_t)d.n;
    d_lab_in = tmp;
  }
  OrientBufs ob;
  orient_carve(ctx, d.n, d.nnz, want_edges, false, bump, ob);
  CountBufs cb;
  if (count_carve(ctx, d.n, d.nnz, bump, cb, o.record_tile_costs != 0) != TC_OK || bump.overflow)
    return set_error(ctx, TC_ERR_OOM, "arena overflow");
  uint8_t *d_lab = bump.take<uint8_t>(d.n);
  uint32_t *d_out = nullptr;
  if (want_edges) d_out = g->on_device ? edge_counts : bump.take<uint32_t>(d.nnz);
  if (bump.overflow) return set_error(ctx, TC_ERR_OOM, "arena overflow");
  int64_t m = 0;
  float ms_a = 0;
  TC_TRY(orient_front(ctx, d, o, ob, &m, &st.ms_validate, &ms_a));
  st.ms_h2d = elapsed(ctx->ev[0], ctx->ev[1]);
  if (want_edges && edge_capacity < m)
    return set_error(ctx, TC_ERR_INVALID_ARG, "edge_counts holds %lld entries, %lld oriented edges",
                     (long long)edge_capacity, (long long)m);
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[4], ctx->stream));
  DevDag dag;
  TC_TRY(orient_phase_b(ctx, d, ob, m, want_edges, false, &dag));
  TC_TRY(launch_relabel_u8(ctx, d_lab_in, ob.rank, d.n, d_lab));
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[5], ctx->stream));
  dag.vlabel = d_lab;
  dag.label = label;
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_total, 0, sizeof(unsigned long long), ctx->stream));
  TC_TRY(run_count(ctx, dag, o, cb, d_out, true));
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[6], ctx->stream));
  if (want_edges && !g->on_device && m > 0) {
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(edge_counts, d_out, sizeof(uint32_t) * (size_t)m, cudaMemcpyDeviceToHost,
                                       ctx->stream));
    st.d2h_bytes += sizeof(uint32_t) * (size_t)m;
  }
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ctx->h_pinned[2], ctx->d_total, sizeof(unsigned long long),
                                     cudaMemcpyDeviceToHost, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ctx->h_pinned[3], ctx->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost,
                                     ctx->stream));
  st.d2h_bytes += sizeof(unsigned long long);
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[7], ctx->stream));
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  TC_TRY(check_wait_flags(ctx));
  *total = ctx->h_pinned[2];
  count_stats(ctx, &st, true);
  st.ms_orient = ms_a + elapsed(ctx->ev[4], ctx->ev[5]);
  st.ms_d2h = elapsed(ctx->ev[6], ctx->ev[7]);
  st.ms_total = elapsed(ctx->ev[0], ctx->ev[7]);
  st.m = m;
  st.tiles = (m + TILE_EDGES - 1) / TILE_EDGES;
  st.kernel_launches = ctx->launches;
  if (stats) *stats = st;
  return TC_OK;
}

// Triangles through every vertex.  Every triangle u < v < w (ranks) is found
// once, on edge u->v with w the hit: the per-edge counts give the lowest
// (u: row sums) and middle (v: in-edge sums) vertex; the PULL arm adds, per
// hit, one to entry u->w (top counts), whose in-edge sums give the highest.
tc_status tc_count_vertices(tc_ctx *ctx, const tc_csr *g, const tc_opts *opts_in, uint64_t *total,
                            uint64_t *vertex_counts, tc_stats *stats) {
  if (!ctx || !total || !vertex_counts) return set_error(ctx, TC_ERR_INVALID_ARG, "null ctx, total or vertex_counts");
  TC_TRY(check_csr_args(ctx, g));
  tc_opts o;
  tc_opts_default(&o);
  if (opts_in) o = *opts_in;
  o.selector = TC_SELECT_FORCE;  // only the PULL arm attributes the top edge of a triangle
  o.force_arm = TC_ARM_PULL;
  TC_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  ctx->launches = 0;
  tc_stats st;
  memset(&st, 0, sizeof(st));
  Sizer sz;
  if (!g->on_device) { sz.take<int64_t>(g->n + 1); sz.take<int32_t>(g->nnz); }
  orient_sizes(ctx, g->n, g->nnz, false, false, sz);
  sz.used += count_scratch_bytes(ctx, g->n, g->nnz);
  sz.take<uint32_t>(g->nnz);
  sz.take<uint32_t>(g->nnz);
  sz.take<unsigned long long>(g->n);
  if (!g->on_device) sz.take<unsigned long long>(g->n);
  TC_TRY(arena_reserve(ctx, sz.used));
  Bump bump{ctx->arena, ctx->arena_cap};
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned) * 8, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
  DevCSR d;
  TC_TRY(stage_csr(ctx, g, bump, d, &st.h2d_bytes));
  OrientBufs ob;
  orient_carve(ctx, d.n, d.nnz, false, false, bump, ob);
  CountBufs cb;
  if (count_carve(ctx, d.n, d.nnz, bump, cb, o.record_tile_costs != 0) != TC_OK || bump.overflow)
    return set_error(ctx, TC_ERR_OOM, "arena overflow");
  uint32_t *d_c = bump.take<uint32_t>(d.nnz);
  uint32_t *d_top = bump.take<uint32_t>(d.nnz);
  unsigned long long *d_t = bump.take<unsigned long long>(d.n);
  unsigned long long *d_vc = g->on_device ? reinterpret_cast<unsigned long long *>(vertex_counts)
                                          : bump.take<unsigned long long>(d.n);
  if (bump.overflow) return set_error(ctx, TC_ERR_OOM, "arena overflow");
  int64_t m = 0;
  float ms_a = 0;
  TC_TRY(orient_front(ctx, d, o, ob, &m, &st.ms_validate, &ms_a));
  st.ms_h2d = elapsed(ctx->ev[0], ctx->ev[1]);
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[4], ctx->stream));
  DevDag dag;
  TC_TRY(orient_phase_b(ctx, d, ob, m, false, false, &dag));
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[5], ctx->stream));
  if (m > 0) TC_CHECK_CUDA(ctx, cudaMemsetAsync(d_top, 0, sizeof(uint32_t) * (size_t)m, ctx->stream));
  dag.top = d_top;
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_total, 0, sizeof(unsigned long long), ctx->stream));
  TC_TRY(run_count(ctx, dag, o, cb, d_c, true));
  TC_TRY(launch_vertex_sums(ctx, dag, d_c, d_top, d_t, ob.rank, d_vc));
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[6], ctx->stream));
  if (!g->on_device && d.n > 0) {
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(vertex_counts, d_vc, sizeof(uint64_t) * (size_t)d.n, cudaMemcpyDeviceToHost,
                                       ctx->stream));
    st.d2h_bytes += sizeof(uint64_t) * (size_t)d.n;
  }
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ctx->h_pinned[2], ctx->d_total, sizeof(unsigned long long),
                                     cudaMemcpyDeviceToHost, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ctx->h_pinned[3], ctx->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost,
                                     ctx->stream));
  st.d2h_bytes += sizeof(unsigned long long);
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[7], ctx->stream));
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  TC_TRY(check_wait_flags(ctx));
  *total = ctx->h_pinned[2];
  count_stats(ctx, &st, true);
  st.ms_orient = ms_a + elapsed(ctx->ev[4], ctx->ev[5]);
  st.ms_d2h = elapsed(ctx->ev[6], ctx->ev[7]);
  st.ms_total = elapsed(ctx->ev[0], ctx->ev[7]);
  st.m = m;
  st.tiles = (m + TILE_EDGES - 1) / TILE_EDGES;
  st.kernel_launches = ctx->launches;
  if (stats) *stats = st;
  return TC_OK;
}

// Partitioned counting on top of tc_count_dag: the graph's part table and
// where the per-partition sums go (host memory).
struct PartReq {
  const int64_t *part;
  int32_t num_parts;
  int32_t rule;
  uint64_t *totals;
};

// Rows [row_begin, row_end) of an oriented graph counted against the whole
// graph (tc_count_dag_range).
struct RangeReq {
  int64_t row_begin, row_end;
};

static tc_status count_dag_impl(tc_ctx *ctx, const tc_csr *dag_in, const tc_opts *opts_in, uint64_t *total,
                                uint32_t *edge_counts, int64_t edge_capacity, tc_stats *stats, const PartReq *pr,
                                const RangeReq *rr = nullptr) {
  if (!ctx || !total) return set_error(ctx, TC_ERR_INVALID_ARG, "null ctx or total");
  TC_TRY(check_csr_args(ctx, dag_in));
  tc_opts o;
  tc_opts_default(&o);
  if (opts_in) o = *opts_in;
  TC_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  ctx->launches = 0;
  tc_stats st;
  memset(&st, 0, sizeof(st));
  const int64_t m = dag_in->nnz;
  // The counted edges: all of them, or the entries of a row range
  // [e0, e1) = [rowptr[row_begin], rowptr[row_end]).
  int64_t e0 = 0, e1 = m;
  if (rr) {
    if (rr->row_begin < 0 || rr->row_begin > rr->row_end || rr->row_end > dag_in->n)
      return set_error(ctx, TC_ERR_INVALID_ARG, "row range [%lld, %lld) outside [0, %lld]", (long long)rr->row_begin,
                       (long long)rr->row_end, (long long)dag_in->n);
    if (dag_in->on_device) {
      TC_CHECK_CUDA(ctx, cudaMemcpy(&e0, dag_in->rowptr + rr->row_begin, sizeof(int64_t), cudaMemcpyDeviceToHost));
      TC_CHECK_CUDA(ctx, cudaMemcpy(&e1, dag_in->rowptr + rr->row_end, sizeof(int64_t), cudaMemcpyDeviceToHost));
    } else {
      e0 = dag_in->rowptr[rr->row_begin];
      e1 = dag_in->rowptr[rr->row_end];
    }
    if (e0 < 0 || e0 > e1 || e1 > m)
      return set_error(ctx, TC_ERR_INVALID_GRAPH, "row pointers of the range [%lld, %lld) are not within [0, nnz]",
                       (long long)rr->row_begin, (long long)rr->row_end);
  }
  const int64_t m_out = e1 - e0;
  const bool want_edges = edge_counts != nullptr;
  if (want_edges && edge_capacity < m_out)
    return set_error(ctx, TC_ERR_INVALID_ARG, "edge_counts holds %lld entries, %lld edges", (long long)edge_capacity,
                     (long long)m_out);
  // partitioned sums need per-edge counts on the device
  const bool dev_edges = want_edges || pr != nullptr;
  Sizer sz;
  if (!dag_in->on_device) { sz.take<int64_t>(dag_in->n + 1); sz.take<int32_t>(m); }
  sz.take<int32_t>(m);
  sz.take<int32_t>(dag_in->n);
  if (rr) sz.take<int64_t>(dag_in->n + 1);
  sz.used += count_scratch_bytes(ctx, dag_in->n, m);
  if (dev_edges && !(want_edges && dag_in->on_device)) sz.take<uint32_t>(m_out);
  if (pr) {
    if (!dag_in->on_device) sz.take<int64_t>(dag_in->n);
    sz.take<unsigned long long>(pr->num_parts);
  }
  TC_TRY(arena_reserve(ctx, sz.used));
  Bump bump{ctx->arena, ctx->arena_cap};
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
  DevCSR d;
  TC_TRY(stage_csr(ctx, dag_in, bump, d, &st.h2d_bytes));
  int32_t *src = bump.take<int32_t>(m);
  int32_t *indeg = bump.take<int32_t>(dag_in->n);
  int64_t *range_rowptr = rr ? bump.take<int64_t>(dag_in->n + 1) : nullptr;
  CountBufs cb;
  if (count_carve(ctx, dag_in->n, m, bump, cb, o.record_tile_costs != 0) != TC_OK || bump.overflow)
    return set_error(ctx, TC_ERR_OOM, "arena overflow");
  uint32_t *d_out = nullptr;
  if (dev_edges) d_out = (want_edges && dag_in->on_device) ? edge_counts : bump.take<uint32_t>(m_out);
  const int64_t *d_part = nullptr;
  unsigned long long *d_pt = nullptr;
  if (pr) {
    if (dag_in->on_device) {
      d_part = pr->part;
    } else {
      int64_t *hp = bump.take<int64_t>(dag_in->n);
      if (bump.overflow) return set_error(ctx, TC_ERR_OOM, "arena overflow");
      TC_CHECK_CUDA(ctx, cudaMemcpyAsync(hp, pr->part, sizeof(int64_t) * (size_t)dag_in->n, cudaMemcpyHostToDevice,
                                         ctx->stream));
      st.h2d_bytes += sizeof(int64_t) * (size_t)dag_in->n;
      d_part = hp;
    }
    d_pt = bump.take<unsigned long long>(pr->num_parts);
    if (bump.overflow) return set_error(ctx, TC_ERR_OOM, "arena overflow");
  }
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned) * 8, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[1], ctx->stream));
  // A DAG row may hold any larger-or-smaller ids; only sortedness is required.
  if (o.validate) TC_TRY(launch_validate(ctx, d, true));
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[2], ctx->stream));
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ctx->h_pinned[1], ctx->d_flags, sizeof(unsigned) * 2, cudaMemcpyDeviceToHost,
                                     ctx->stream));
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const unsigned flags = (unsigned)(ctx->h_pinned[1] & 0xffffffffu);
  if (flags) return set_error(ctx, TC_ERR_INVALID_GRAPH, "%s", flag_text(flags));
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[4], ctx->stream));
  TC_TRY(launch_expand_src(ctx, d.rowptr, d.n, m, src));
  TC_TRY(launch_indeg(ctx, d.col, d.n, m, indeg));
  // A row range is counted in place: its edges are entries [e0, e1) of the
  // column array, so the count runs on col + e0 with row pointers shifted by
  // -e0 (every row's list, inside the range or not, stays where it is).
  if (rr) TC_TRY(launch_shift_rowptr(ctx, d.rowptr, d.n, e0, range_rowptr));
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[5], ctx->stream));
  DevDag dag;
  dag.n = d.n;
  dag.m = m_out;
  dag.rowptr = rr ? range_rowptr : d.rowptr;
  dag.col = d.col + e0;
  dag.src = src + e0;
  dag.perm = nullptr;
  dag.indeg = indeg;
  dag.restrict_after = 0;
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_total, 0, sizeof(unsigned long long), ctx->stream));
  TC_TRY(run_count(ctx, dag, o, cb, d_out, true));
  if (pr) TC_TRY(launch_part_sums(ctx, dag, d_out, d_part, pr->num_parts, pr->rule, d_pt));
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[6], ctx->stream));
  if (want_edges && !dag_in->on_device && m_out > 0) {
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(edge_counts, d_out, sizeof(uint32_t) * (size_t)m_out, cudaMemcpyDeviceToHost,
                                       ctx->stream));
    st.d2h_bytes += sizeof(uint32_t) * (size_t)m_out;
  }
  if (pr) {
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(pr->totals, d_pt, sizeof(uint64_t) * (size_t)pr->num_parts,
                                       cudaMemcpyDeviceToHost, ctx->stream));
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ctx->h_pinned[1], ctx->d_flags, sizeof(unsigned) * 2, cudaMemcpyDeviceToHost,
                                       ctx->stream));
    st.d2h_bytes += sizeof(uint64_t) * (size_t)pr->num_parts;
  }
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ctx->h_pinned[2], ctx->d_total, sizeof(unsigned long long),
                                     cudaMemcpyDeviceToHost, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ctx->h_pinned[3], ctx->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost,
                                     ctx->stream));
  st.d2h_bytes += sizeof(unsigned long long);
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[7], ctx->stream));
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (pr && (ctx->h_pinned[1] & VF_PART_RANGE))
    return set_error(ctx, TC_ERR_INVALID_ARG, "%s", flag_text(VF_PART_RANGE));
  TC_TRY(check_wait_flags(ctx));
  *total = ctx->h_pinned[2];
  count_stats(ctx, &st, true);
  st.ms_h2d = elapsed(ctx->ev[0], ctx->ev[1]);
  st.ms_validate = elapsed(ctx->ev[1], ctx->ev[2]);
  st.ms_orient = elapsed(ctx->ev[4], ctx->ev[5]);
  st.ms_d2h = elapsed(ctx->ev[6], ctx->ev[7]);
  st.ms_total = elapsed(ctx->ev[0], ctx->ev[7]);
  st.m = m_out;
  st.tiles = (m_out + TILE_EDGES - 1) / TILE_EDGES;
  st.kernel_launches = ctx->launches;
  if (stats) *stats = st;
  return TC_OK;
}

tc_status tc_count_dag(tc_ctx *ctx, const tc_csr *dag_in, const tc_opts *opts_in, uint64_t *total,
                       uint32_t *edge_counts, int64_t edge_capacity, tc_stats *stats) {
  return count_dag_impl(ctx, dag_in, opts_in, total, edge_counts, edge_capacity, stats, nullptr);
}

tc_status tc_count_dag_range(tc_ctx *ctx, const tc_csr *dag, int64_t row_begin, int64_t row_end,
                             const tc_opts *opts, uint64_t *total, uint32_t *edge_counts, int64_t edge_capacity,
                             tc_stats *stats) {
  const RangeReq rr{row_begin, row_end};
  return count_dag_impl(ctx, dag, opts, total, edge_counts, edge_capacity, stats, nullptr, &rr);
}

tc_status tc_count_dag_parts(tc_ctx *ctx, const tc_csr *dag, const int64_t *part, int32_t num_parts, int32_t rule,
                             const tc_opts *opts, uint64_t *total, uint64_t *part_totals, tc_stats *stats) {
  if (!ctx) return set_error(ctx, TC_ERR_INVALID_ARG, "null ctx");
  if (!part || !part_totals || num_parts < 1)
    return set_error(ctx, TC_ERR_INVALID_ARG, "null part or part_totals, or num_parts=%d < 1", (int)num_parts);
  if (rule != TC_PART_BY_SOURCE && rule != TC_PART_PUSH_PULL)
    return set_error(ctx, TC_ERR_INVALID_ARG, "unknown partition rule %d", (int)rule);
  const PartReq pr{part, num_parts, rule, part_totals};
  return count_dag_impl(ctx, dag, opts, total, nullptr, 0, stats, &pr);
}

tc_status tc_orient(tc_ctx *ctx, const tc_csr *g, int64_t *dag_rowptr, int32_t *dag_colidx, int64_t dag_capacity,
                    int64_t *m_out) {
  if (!ctx || !dag_rowptr || !m_out) return set_error(ctx, TC_ERR_INVALID_ARG, "null argument");
  TC_TRY(check_csr_args(ctx, g));
  tc_opts o;
  tc_opts_default(&o);
  TC_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  ctx->launches = 0;
  Sizer sz;
  if (!g->on_device) { sz.take<int64_t>(g->n + 1); sz.take<int32_t>(g->nnz); }
  orient_sizes(ctx, g->n, g->nnz, false, true, sz);
  if (!g->on_device) sz.take<int64_t>(g->n + 1);
  TC_TRY(arena_reserve(ctx, sz.used));
  Bump bump{ctx->arena, ctx->arena_cap};
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned) * 8, ctx->stream));
  uint64_t h2d = 0;
  DevCSR d;
  TC_TRY(stage_csr(ctx, g, bump, d, &h2d));
  OrientBufs ob;
  orient_carve(ctx, d.n, d.nnz, false, true, bump, ob);
  int64_t *d_rp = g->on_device ? dag_rowptr : bump.take<int64_t>(g->n + 1);
  if (bump.overflow) return set_error(ctx, TC_ERR_OOM, "arena overflow");
  int64_t m = 0;
  float a, b;
  TC_TRY(orient_front(ctx, d, o, ob, &m, &a, &b));
  *m_out = m;
  if (m > dag_capacity || (m > 0 && !dag_colidx))
    return set_error(ctx, TC_ERR_INVALID_ARG, "dag_colidx holds %lld entries, %lld needed", (long long)dag_capacity,
                     (long long)m);
  if (g->on_device) ob.dag_col = dag_colidx;
  DevDag dag;
  (void)dag;
  TC_TRY(orient_phase_b(ctx, d, ob, m, false, true, nullptr));  // original-id columns only, no relabel
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(d_rp, ob.orowptr, sizeof(int64_t) * (size_t)(d.n + 1), cudaMemcpyDeviceToDevice,
                                     ctx->stream));
  if (!g->on_device) {
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(dag_rowptr, d_rp, sizeof(int64_t) * (size_t)(d.n + 1), cudaMemcpyDeviceToHost,
                                       ctx->stream));
    if (m > 0)
      TC_CHECK_CUDA(ctx, cudaMemcpyAsync(dag_colidx, ob.dag_col, sizeof(int32_t) * (size_t)m, cudaMemcpyDeviceToHost,
                                         ctx->stream));
  }
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TC_OK;
}

}  // extern "C"
