// Batched counting of many small graphs and per-tile profiling for the
// learned selector.
//
// A batch is counted as the disjoint union of its graphs: local ids become
// global ids, every vertex carries its graph as a rank-key group, so each
// graph owns a contiguous range of ranks and therefore of relabelled edges;
// the count kernels pull (graph, tile) items from the per-arm queues of that
// one union graph and a segmented sum yields every graph's exact total.  The
// orientation's front half (up to the host read of the oriented edge count)
// and the back half -> count -> per-graph-sum pipeline are each captured once
// as a CUDA graph per batch shape and replayed.
#include <algorithm>
#include <vector>

#include "engine.cuh"

using namespace tc;

namespace tc {

constexpr int BT_THREADS = 256;

__global__ void group_fill_kernel(const int64_t *__restrict__ vtx_off, int64_t G, int64_t n,
                                  int32_t *__restrict__ vgroup, unsigned *flags) {
  for (int64_t g = blockIdx.x; g < G; g += gridDim.x) {
    const int64_t a = vtx_off[g], b = vtx_off[g + 1];
    if (b < a || a < 0 || b > n) {
      if (threadIdx.x == 0) atomicOr(flags, (unsigned)VF_ROWPTR_ORDER);
      continue;
    }
    for (int64_t v = a + threadIdx.x; v < b; v += blockDim.x) vgroup[v] = (int32_t)g;
  }
}

// Graph g owns relabelled rows [vtx_off[g], vtx_off[g+1]) and so the edge
// range [nrowptr[vtx_off[g]], nrowptr[vtx_off[g+1]]).
__global__ void __launch_bounds__(BT_THREADS) graph_sum_kernel(const uint32_t *__restrict__ cnt,
                                                              const int64_t *__restrict__ nrowptr,
                                                              const int64_t *__restrict__ vtx_off, int64_t G,
                                                              unsigned long long *__restrict__ totals) {
  __shared__ unsigned long long part[BT_THREADS / 32];
  for (int64_t g = blockIdx.x; g < G; g += gridDim.x) {
    const int64_t a = nrowptr[vtx_off[g]], b = nrowptr[vtx_off[g + 1]];
    unsigned long long s = 0;
    for (int64_t e = a + threadIdx.x; e < b; e += BT_THREADS) s += cnt[e];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long t = 0;
      for (int w = 0; w < BT_THREADS / 32; ++w) t += part[w];
      totals[g] = t;
    }
    __syncthreads();
  }
}

}  // namespace tc

extern "C" {

tc_status tc_batch_count(tc_ctx *ctx, const tc_batch *b, const tc_opts *opts_in, uint64_t *totals, tc_stats *stats) {
  if (!ctx || !b || !totals || b->num_graphs < 1 || !b->vtx_off || !b->rowptr)
    return set_error(ctx, TC_ERR_INVALID_ARG, "bad batch arguments");
  tc_opts o;
  tc_opts_default(&o);
  if (opts_in) o = *opts_in;
  TC_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  ctx->launches = 0;
  tc_stats st;
  memset(&st, 0, sizeof(st));
  const int64_t G = b->num_graphs;
  int64_t n = 0, nnz = 0;
  if (b->on_device) {
    TC_CHECK_CUDA(ctx, cudaMemcpy(&n, b->vtx_off + G, sizeof(int64_t), cudaMemcpyDeviceToHost));
    if (n < 1 || n > 2147483647LL) return set_error(ctx, TC_ERR_UNSUPPORTED, "batch holds %lld vertices", (long long)n);
    TC_CHECK_CUDA(ctx, cudaMemcpy(&nnz, b->rowptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost));
  } else {
    n = b->vtx_off[G];
    if (b->vtx_off[0] != 0 || n < 1 || n > 2147483647LL)
      return set_error(ctx, TC_ERR_UNSUPPORTED, "batch vertex offsets must start at 0 and hold [1, 2^31) vertices");
    nnz = b->rowptr[n];
  }
  if (nnz < 0 || nnz >= (int64_t(1) << 32) || (nnz > 0 && !b->colidx))
    return set_error(ctx, TC_ERR_UNSUPPORTED, "batch nnz=%lld outside [0, 2^32)", (long long)nnz);
  const int gbits = bit_width_u64((uint64_t)(G > 1 ? G - 1 : 1));
  Sizer sz;
  if (!b->on_device) { sz.take<int64_t>(G + 1); sz.take<int64_t>(n + 1); sz.take<int32_t>(nnz); }
  sz.take<int32_t>(n);
  orient_sizes(ctx, n, nnz, false, false, sz);
  sz.used += count_scratch_bytes(ctx, n, nnz);
  sz.take<uint32_t>(nnz);
  sz.take<unsigned long long>(G);
  TC_TRY(arena_reserve(ctx, sz.used));
  Bump bump{ctx->arena, ctx->arena_cap};
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
  const int64_t *d_off = b->vtx_off, *d_row = b->rowptr;
  const int32_t *d_col = b->colidx;
  if (!b->on_device) {
    int64_t *o1 = bump.take<int64_t>(G + 1), *r1 = bump.take<int64_t>(n + 1);
    int32_t *c1 = bump.take<int32_t>(nnz);
    if (bump.overflow) return set_error(ctx, TC_ERR_OOM, "arena overflow");
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(o1, b->vtx_off, sizeof(int64_t) * (G + 1), cudaMemcpyHostToDevice, ctx->stream));
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(r1, b->rowptr, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, ctx->stream));
    if (nnz > 0)
      TC_CHECK_CUDA(ctx, cudaMemcpyAsync(c1, b->colidx, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, ctx->stream));
    st.h2d_bytes = sizeof(int64_t) * (G + 1 + n + 1) + sizeof(int32_t) * nnz;
    d_off = o1;
    d_row = r1;
    d_col = c1;
  }
  int32_t *vgroup = bump.take<int32_t>(n);
  OrientBufs ob;
  orient_carve(ctx, n, nnz, false, false, bump, ob);
  ob.vgroup = vgroup;
  ob.group_bits = gbits;
  ob.vtx_off = d_off;
  CountBufs cb;
  if (count_carve(ctx, n, nnz, bump, cb, false) != TC_OK) return set_error(ctx, TC_ERR_OOM, "arena overflow");
  uint32_t *cnt = bump.take<uint32_t>(nnz);
  unsigned long long *d_tot = bump.take<unsigned long long>(G);
  if (bump.overflow) return set_error(ctx, TC_ERR_OOM, "arena overflow");
  DevCSR d;  // local column ids: the kept-count pass adds each row's graph base (ob.vtx_off)
  d.n = n;
  d.nnz = nnz;
  d.rowptr = d_row;
  d.col = d_col;
  // Front half (graph ids, validation, rank sort, kept counts, scans and the
  // queued copies of m and the flags), replayed as a CUDA graph when the
  // batch shape and buffers repeat; the host then reads m and the flags.
  const int64_t fkey[12] = {n, nnz, G, o.validate, (int64_t)(uintptr_t)ctx->arena, (int64_t)ctx->arena_cap,
                            (int64_t)(uintptr_t)d_col, (int64_t)(uintptr_t)d_row, (int64_t)(uintptr_t)d_off,
                            (int64_t)b->on_device, ctx->orient_blocks_per_sm, 0};
  const bool fsame = ctx->batch_front_exec && memcmp(fkey, ctx->batch_front_key, sizeof(fkey)) == 0;
  if (!fsame) {
    if (ctx->batch_front_exec) {
      cudaGraphExecDestroy(ctx->batch_front_exec);
      ctx->batch_front_exec = nullptr;
    }
    const int64_t launches0 = ctx->launches;
    cudaGraph_t graph;
    TC_CHECK_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    tc_status s0 = TC_OK;
    if (cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned) * 8, ctx->stream) != cudaSuccess ||
        cudaMemsetAsync(vgroup, 0, sizeof(int32_t) * n, ctx->stream) != cudaSuccess)
      s0 = set_error(ctx, TC_ERR_CUDA, "memset during capture failed");
    if (s0 == TC_OK) {
      group_fill_kernel<<<(int)std::min<int64_t>(G, 65535), 256, 0, ctx->stream>>>(d_off, G, n, vgroup,
                                                                                  ctx->d_flags);
      ctx->launches++;
      s0 = orient_front_launch(ctx, d, o, ob);
    }
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
    if (s0 != TC_OK) {
      if (ce == cudaSuccess) cudaGraphDestroy(graph);
      return s0;
    }
    TC_CHECK_CUDA(ctx, ce);
    cudaError_t ie = cudaGraphInstantiate(&ctx->batch_front_exec, graph, 0);
    cudaGraphDestroy(graph);
    TC_CHECK_CUDA(ctx, ie);
    memcpy(ctx->batch_front_key, fkey, sizeof(fkey));
    ctx->batch_front_launches = ctx->launches - launches0;
  } else {
    ctx->launches += ctx->batch_front_launches;
  }
  TC_CHECK_CUDA(ctx, cudaGraphLaunch(ctx->batch_front_exec, ctx->stream));
  int64_t m = 0;
  float ms_a = 0;
  TC_TRY(orient_front_finish(ctx, &m, &st.ms_validate, &ms_a));
  // Back half (relabel sort -> count -> per-graph sums -> D2H), replayed as
  // a CUDA graph when the batch shape and buffers repeat.
  const int64_t key[14] = {n, nnz, m, G, o.selector, o.force_arm, (int64_t)(uintptr_t)ctx->arena,
                           (int64_t)ctx->arena_cap, (int64_t)(uintptr_t)d_col, (int64_t)(uintptr_t)d_row,
                           (int64_t)(uintptr_t)d_off, (int64_t)ctx->mlp_loaded,
                           ((int64_t)ctx->pull_item << 32) | (uint32_t)ctx->pull_item_min,
                           ((int64_t)ctx->pull_block_tiles << 32) | (ctx->pull_dense_num << 16) | ctx->pull_dense_den};
  const bool same = ctx->batch_exec && memcmp(key, ctx->batch_key, sizeof(key)) == 0;
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[4], ctx->stream));
  if (!same) {
    if (ctx->batch_exec) {
      cudaGraphExecDestroy(ctx->batch_exec);
      ctx->batch_exec = nullptr;
    }
    const int64_t launches0 = ctx->launches;
    cudaGraph_t graph;
    TC_CHECK_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    DevDag dag;
    tc_status s1 = orient_phase_b(ctx, d, ob, m, false, false, &dag);
    if (s1 == TC_OK) {
      cudaMemsetAsync(ctx->d_total, 0, sizeof(unsigned long long), ctx->stream);
      s1 = run_count(ctx, dag, o, cb, cnt, false);
    }
    if (s1 == TC_OK) {
      graph_sum_kernel<<<(int)std::min<int64_t>(G, 65535), BT_THREADS, 0, ctx->stream>>>(cnt, ob.nrowptr, d_off, G,
                                                                                         d_tot);
      ctx->launches++;
    }
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
    if (s1 != TC_OK) {
      if (ce == cudaSuccess) cudaGraphDestroy(graph);
      return s1;
    }
    TC_CHECK_CUDA(ctx, ce);
    cudaError_t ie = cudaGraphInstantiate(&ctx->batch_exec, graph, 0);
    cudaGraphDestroy(graph);
    TC_CHECK_CUDA(ctx, ie);
    memcpy(ctx->batch_key, key, sizeof(key));
    ctx->batch_launches = ctx->launches - launches0;
  } else {
    ctx->launches += ctx->batch_launches;
  }
  TC_CHECK_CUDA(ctx, cudaGraphLaunch(ctx->batch_exec, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[6], ctx->stream));
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(totals, d_tot, sizeof(unsigned long long) * G, cudaMemcpyDeviceToHost,
                                     ctx->stream));
  st.d2h_bytes = sizeof(unsigned long long) * G;
  TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[7], ctx->stream));
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  count_stats(ctx, &st, false);
  st.ms_h2d = elapsed(ctx->ev[0], ctx->ev[1]);
  st.ms_orient = ms_a;
  st.ms_count = elapsed(ctx->ev[4], ctx->ev[6]);  // relabel sort + count + sums (one graph launch)
  st.ms_d2h = elapsed(ctx->ev[6], ctx->ev[7]);
  st.ms_total = elapsed(ctx->ev[0], ctx->ev[7]);
  st.m = m;
  st.tiles = (m + TILE_EDGES - 1) / TILE_EDGES;
  st.kernel_launches = ctx->launches;
  if (stats) *stats = st;
  return TC_OK;
}

tc_status tc_plan_arms(tc_ctx *ctx, const tc_csr *g, const tc_opts *opts_in, int32_t *arms, int64_t capacity,
                       int64_t *tiles_out) {
  if (!ctx || !g || !tiles_out) return set_error(ctx, TC_ERR_INVALID_ARG, "null argument");
  if (g->n < 1 || g->n > 2147483647LL || g->nnz < 0 || g->nnz >= (int64_t(1) << 32) || !g->rowptr ||
      (g->nnz > 0 && !g->colidx))
    return set_error(ctx, TC_ERR_INVALID_ARG, "bad graph");
  tc_opts o;
  tc_opts_default(&o);
  if (opts_in) o = *opts_in;
  TC_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  ctx->launches = 0;
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned) * 8, ctx->stream));
  Sizer sz;
  if (!g->on_device) { sz.take<int64_t>(g->n + 1); sz.take<int32_t>(g->nnz); }
  orient_sizes(ctx, g->n, g->nnz, false, false, sz);
  sz.used += count_scratch_bytes(ctx, g->n, g->nnz);
  TC_TRY(arena_reserve(ctx, sz.used));
  Bump bump{ctx->arena, ctx->arena_cap};
  uint64_t h2d = 0;
  DevCSR d;
  TC_TRY(stage_csr(ctx, g, bump, d, &h2d));
  OrientBufs ob;
  orient_carve(ctx, d.n, d.nnz, false, false, bump, ob);
  CountBufs cb;
  if (count_carve(ctx, d.n, d.nnz, bump, cb, false) != TC_OK || bump.overflow) return set_error(ctx, TC_ERR_OOM, "arena");
  int64_t m = 0;
  float a, bb;
  TC_TRY(orient_front(ctx, d, o, ob, &m, &a, &bb));
  DevDag dag;
  TC_TRY(orient_phase_b(ctx, d, ob, m, false, false, &dag));
  const int64_t T = (m + TILE_EDGES - 1) / TILE_EDGES;
  *tiles_out = T;
  if (T > capacity || (T > 0 && !arms))
    return set_error(ctx, TC_ERR_INVALID_ARG, "arms holds %lld tiles, %lld needed", (long long)capacity,
                     (long long)T);
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_total, 0, sizeof(unsigned long long), ctx->stream));
  TC_TRY(run_count(ctx, dag, o, cb, nullptr, false));
  if (T > 0)
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(arms, cb.arm, sizeof(int32_t) * T, cudaMemcpyDeviceToHost, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TC_OK;
}

tc_status tc_tile_profile(tc_ctx *ctx, const tc_csr *g, float *features, float *costs, int64_t capacity,
                          int64_t *tiles_out) {
  if (!ctx || !g || !tiles_out) return set_error(ctx, TC_ERR_INVALID_ARG, "null argument");
  if (g->n < 1 || g->n > 2147483647LL || g->nnz < 0 || g->nnz >= (int64_t(1) << 32) || !g->rowptr ||
      (g->nnz > 0 && !g->colidx))
    return set_error(ctx, TC_ERR_INVALID_ARG, "bad graph");
  TC_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
  ctx->launches = 0;
  tc_opts o;
  tc_opts_default(&o);
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned) * 8, ctx->stream));
  Sizer sz;
  if (!g->on_device) { sz.take<int64_t>(g->n + 1); sz.take<int32_t>(g->nnz); }
  orient_sizes(ctx, g->n, g->nnz, false, false, sz);
  sz.used += count_scratch_bytes(ctx, g->n, g->nnz);
  TC_TRY(arena_reserve(ctx, sz.used));
  Bump bump{ctx->arena, ctx->arena_cap};
  uint64_t h2d = 0;
  DevCSR d;
  TC_TRY(stage_csr(ctx, g, bump, d, &h2d));
  OrientBufs ob;
  orient_carve(ctx, d.n, d.nnz, false, false, bump, ob);
  CountBufs cb;
  if (count_carve(ctx, d.n, d.nnz, bump, cb, true) != TC_OK || bump.overflow) return set_error(ctx, TC_ERR_OOM, "arena");
  int64_t m = 0;
  float a, bb;
  TC_TRY(orient_front(ctx, d, o, ob, &m, &a, &bb));
  DevDag dag;
  TC_TRY(orient_phase_b(ctx, d, ob, m, false, false, &dag));
  const int64_t T = (m + TILE_EDGES - 1) / TILE_EDGES;
  *tiles_out = T;
  if (T > capacity || (T > 0 && (!features || !costs)))
    return set_error(ctx, TC_ERR_INVALID_ARG, "buffers hold %lld tiles, %lld needed", (long long)capacity,
                     (long long)T);
  std::vector<unsigned long long> cyc((size_t)T);
  uint64_t first_total = 0;
  for (int arm = 0; arm < TC_NUM_ARMS; ++arm) {
    tc_opts fo = o;
    fo.selector = TC_SELECT_FORCE;
    fo.force_arm = arm;
    TC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_total, 0, sizeof(unsigned long long), ctx->stream));
    TC_TRY(run_count(ctx, dag, fo, cb, nullptr, false));
    if (T > 0)
      TC_CHECK_CUDA(ctx, cudaMemcpyAsync(cyc.data(), cb.tile_cycles, sizeof(unsigned long long) * T,
                                         cudaMemcpyDeviceToHost, ctx->stream));
    if (arm == 0 && T > 0)
      TC_CHECK_CUDA(ctx, cudaMemcpyAsync(features, cb.features, sizeof(float) * T * TC_MLP_FEATURES,
                                         cudaMemcpyDeviceToHost, ctx->stream));
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ctx->h_pinned[2], ctx->d_total, sizeof(unsigned long long),
                                       cudaMemcpyDeviceToHost, ctx->stream));
    TC_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (arm == 0) first_total = ctx->h_pinned[2];
    else if (ctx->h_pinned[2] != first_total)
      return set_error(ctx, TC_ERR_CUDA, "arm %d counted %llu triangles, arm 0 counted %llu", arm,
                       (unsigned long long)ctx->h_pinned[2], (unsigned long long)first_total);
    const float occ = (float)ctx->arm_units_per_sm[arm];  // SM-cycles per tile
    for (int64_t t = 0; t < T; ++t) costs[t * TC_NUM_ARMS + arm] = (float)cyc[(size_t)t] / occ;
  }
  return TC_OK;
}

}  // extern "C"
