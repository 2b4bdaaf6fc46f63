// Triangle counting over an oriented graph: per-edge |N+(u) n N+(v)|.
//
// Work is cut into 4096-edge tiles.  A planning pass computes per-tile
// degree features and picks an exact intersection strategy ("arm") for each
// tile, either with fixed degree thresholds or with the MLP cost model.
// Tiles are radix-sorted into one queue per arm (heaviest first) and each
// arm runs as a persistent kernel whose blocks pull tiles with an atomic
// head, so load balance does not depend on the launch grid.
//
// Arms (all exact; they replace the reference's warp_vertex +
// intersect_num, bs_warp_vertex.cuh:13-21, graph_gpu.h:228-252):
//   BSEARCH_G  G lanes per edge; each lane binary-searches keys of the
//              shorter list in the longer one (the reference's warp_intersect
//              pattern, with the search window carried between keys).
//   MERGE_G    G lanes per edge walk both lists in G-wide windows; each lane
//              locates its A element in the B window with log2(G) shuffles;
//              the window with the smaller last element advances.
//   BITMAP     a block stages the row's remaining out-list as a bitmap over
//              its id window in shared memory and probes every N+(v) against
//              it; rows whose window does not fit fall back to warp search.
#include "engine.cuh"

namespace tc {

constexpr int CT_THREADS = 256;
constexpr int BM_THREADS = 512;
constexpr int BM_SMEM_BYTES = 100 * 1024;
constexpr int64_t BM_BITS = (int64_t)BM_SMEM_BYTES * 8;
constexpr int PLAN_THREADS = 256;
// 1: the planner visits tiles interleaved over the PULL source blocks, so
// the SMs' histogram atomics at any moment go to different blocks' hub keys
// instead of all to the hot hubs of one block (R-MAT scale 24: plan 3.88 ->
// 2.80 ms).  The scatter keeps tile order (PL_SCATTER_INTERLEAVE 0): the
// records of a target group then follow the rows' order, which the probing
// kernel's suffix loads profit from; interleaved tile by tile, or in chunks
// of 64 or 256 tiles, the PULL arm took 1.3, 1.4 and 1.7 ms longer.
#ifndef TC_PL_INTERLEAVE
#define TC_PL_INTERLEAVE 1
#endif
constexpr bool PL_INTERLEAVE = TC_PL_INTERLEAVE != 0;
#ifndef TC_PL_SCATTER_INTERLEAVE
#define TC_PL_SCATTER_INTERLEAVE 0
#endif
constexpr bool PL_SCATTER_INTERLEAVE = TC_PL_SCATTER_INTERLEAVE != 0;
#ifndef TC_PL_SCATTER_GRAIN
#define TC_PL_SCATTER_GRAIN 1
#endif
constexpr int64_t PL_SCATTER_GRAIN = TC_PL_SCATTER_GRAIN;  // tiles per interleaved chunk of the scatter
#ifndef TC_PLAN_UNROLL
#define TC_PLAN_UNROLL 2
#endif
constexpr int PLAN_UNROLL = TC_PLAN_UNROLL;  // plan_kernel: edges per lane with their gathers in flight

// ---- plan: features + selection ------------------------------------------------

struct PlanStats {
  float mean_da, mean_db, mean_min, mean_max;
  float mean_in;  // mean DAG in-degree of the edges' targets
  float alr;  // mean |log2 ratio| of the two list lengths
  float nrows, maxdr, maxwin, frac;
  float bins[6];
};

__device__ __forceinline__ float flog2p1(float x) { return __log2f(1.0f + x); }

// Fixed degree-threshold selector: the engine's default, its fallback, and
// the baseline the learned selector is measured against.
__device__ __forceinline__ int fixed_select(const PlanStats &s) {
  // Thresholds fitted to per-tile arm costs recorded on R-MAT scale 16-20
  // graphs (the learned selector's training set).  The bitmap is cleared per
  // row segment, so it only pays for small id windows.
  // PULL when many edges share each target list (its table build is spread
  // over them) and the lists are long enough for searches to cost more than
  // one shared-memory test per row-suffix entry.
  if (s.mean_in >= 256.f && s.mean_db >= 32.f && s.mean_da >= 8.f) return TC_ARM_PULL;
  if (s.nrows <= 16.f && s.mean_min >= 64.f && s.maxwin <= 16384.f) return TC_ARM_BITMAP;
  if (s.mean_min >= 64.f) return TC_ARM_BSEARCH_32;
  // Lists of similar length (mean |log2 ratio| <= 2.5, e.g. small ER, RGG
  // and R-MAT graphs): an even merge-path split beats searching the longer
  // list; fitted to per-tile costs of R-MAT and of mixed small-graph batches.
  if (s.alr <= 2.5f) return TC_ARM_MPATH_2;
  return TC_ARM_BSEARCH_4;
}

// MLP cost model (16 -> 64 -> 64 -> arms, ReLU); weights staged in shared
// memory rounded to bf16, fp32 accumulation.  Returns the arm with the lowest
// predicted cost.
// The arm of lowest predicted cost, `exclude` (an arm, or -1) left out; it
// replaces `keep` only when predicted at least `margin` (log2 cost) cheaper.
__device__ int mlp_select(const float *__restrict__ w, const float *f, int lane, int exclude, int keep,
                          float margin) {
  const float *W1 = w, *b1 = W1 + TC_MLP_FEATURES * TC_MLP_HIDDEN;
  const float *W2 = b1 + TC_MLP_HIDDEN, *b2 = W2 + TC_MLP_HIDDEN * TC_MLP_HIDDEN;
  const float *W3 = b2 + TC_MLP_HIDDEN, *b3 = W3 + TC_MLP_HIDDEN * TC_NUM_ARMS;
  float h1[2], h2[2];
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int j = lane + 32 * q;
    float a = b1[j];
#pragma unroll
    for (int i = 0; i < TC_MLP_FEATURES; ++i) a = fmaf(f[i], W1[i * TC_MLP_HIDDEN + j], a);
    h1[q] = fmaxf(a, 0.f);
  }
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int j = lane + 32 * q;
    float a = b2[j];
    for (int i = 0; i < TC_MLP_HIDDEN; ++i) {
      const float hi = __shfl_sync(TC_FULL_MASK, h1[i >> 5], i & 31);
      a = fmaf(hi, W2[i * TC_MLP_HIDDEN + j], a);
    }
    h2[q] = fmaxf(a, 0.f);
  }
  int best = -1;
  float bestv = 0.f, keepv = 0.f;
#pragma unroll
  for (int k = 0; k < TC_NUM_ARMS; ++k) {
    float p = h2[0] * W3[lane * TC_NUM_ARMS + k] + h2[1] * W3[(lane + 32) * TC_NUM_ARMS + k];
    p = warp_sum(p) + b3[k];
    if (k == keep) keepv = p;
    if (k == exclude) continue;
    if (best < 0 || p < bestv) { bestv = p; best = k; }
  }
  return (keep >= 0 && keep != exclude && keepv - bestv < margin) ? keep : best;
}

// Grouping key of the PULL arm's counting sort (see the PULL section).
// Hub targets (the top hub_span ids) are grouped per source block of
// block_edges edges, key block * hub_span + (v - hub0); every other target
// per source block of low_block_edges edges, key global0 + block * hub0 + v
// (one such block when TC_PL_WIDE_BLOCKS is 0).
struct PullKeys {
  int64_t hub0;             // first hub id: n - min(n, hub_span)
  int64_t hub_span;         // hub ids, one key per (source block, hub)
  int64_t block_edges;      // edges per source block of the hub part
  int64_t global0;          // first key of the non-hub part: blocks * hub_span
  int64_t low_block_edges;  // edges per source block of the non-hub part
  // key of an edge u->v of tile t (a tile lies in one block of each part):
  // key_in(block_base(t), low_base(t), v)
  __device__ __forceinline__ int64_t block_base(int64_t t) const {
    return (t * TILE_EDGES / block_edges) * hub_span - hub0;
  }
  __device__ __forceinline__ int64_t low_base(int64_t t) const {
    return global0 + (t * TILE_EDGES / low_block_edges) * hub0;
  }
  __device__ __forceinline__ int64_t key_in(int64_t base, int64_t lbase, int32_t v) const {
    return v >= hub0 ? base + v : lbase + v;
  }
};

// One warp per tile: features, the arm, the queue key and the algorithmic
// bytes; a tile that goes to PULL also adds its edges' grouping keys to the
// PULL histogram while its columns are still in cache.
__global__ void __launch_bounds__(PLAN_THREADS) plan_kernel(DevDag g, int64_t T, int selector, int force_arm,
                                                           const float *__restrict__ mlp, float *__restrict__ feats,
                                                           int32_t *__restrict__ arm_out,
                                                           uint64_t *__restrict__ qkeys,
                                                           uint32_t *__restrict__ qvals,
                                                           unsigned long long *__restrict__ tile_bytes,
                                                           PullKeys pk, unsigned *__restrict__ pull_cnt,
                                                           float margin) {
  extern __shared__ float s_w[];
  const int lane = threadIdx.x & 31;
  if (selector == TC_SELECT_LEARNED) {
    for (int i = threadIdx.x; i < TC_MLP_PARAM_COUNT; i += blockDim.x)
      s_w[i] = __bfloat162float(__float2bfloat16(mlp[i]));
    __syncthreads();
  }
  // tiles interleaved over the PULL source blocks (see PL_INTERLEAVE): the
  // grid covers S * per slots, some past the last tile
  const int64_t per = pk.block_edges / TILE_EDGES, S = (T + per - 1) / per;
  const int64_t i = (int64_t)blockIdx.x * (PLAN_THREADS / 32) + (threadIdx.x >> 5);
  const bool lv = PL_INTERLEAVE && S > 1;
  const int64_t t = lv ? (i % S) * per + i / S : i;
  if (i >= (lv ? S * per : T) || t >= T) return;
  const int64_t e0 = t * TILE_EDGES, e1 = min(g.m, e0 + TILE_EDGES);
  float sda = 0, sdb = 0, smin = 0, smax = 0, salr = 0, sin = 0;
  float bins[6] = {0, 0, 0, 0, 0, 0};
  unsigned long long work = 0, alg = 0;
  int nrows = 0;
  long long maxdr = 0, maxwin = 0;
  // PLAN_UNROLL edges per lane at a time, their loads in three rounds, each
  // round's loads all in flight: (row, target, previous edge's row); (row
  // pointers, target degrees); for an edge that starts its row in the tile,
  // the two ends of its row window
  for (int64_t eb = e0 + lane; eb < e1; eb += 32 * PLAN_UNROLL) {
    int32_t rr[PLAN_UNROLL], ss[PLAN_UNROLL], pr[PLAN_UNROLL];
#pragma unroll
    for (int u = 0; u < PLAN_UNROLL; ++u) {
      const int64_t e = eb + 32 * u;
      rr[u] = e < e1 ? g.src[e] : 0;
      ss[u] = e < e1 ? g.col[e] : 0;
      pr[u] = e < e1 && e > e0 ? g.src[e - 1] : -1;
    }
    int64_t rbs[PLAN_UNROLL], res[PLAN_UNROLL];
    int2 dq[PLAN_UNROLL];
#pragma unroll
    for (int u = 0; u < PLAN_UNROLL; ++u) {
      const bool in = eb + 32 * u < e1;
      rbs[u] = in ? g.rowptr[rr[u]] : 0;
      res[u] = in ? g.rowptr[rr[u] + 1] : 0;
      if (!in) dq[u] = make_int2(0, 0);
      else if (g.dv) dq[u] = __ldg(g.dv + ss[u]);  // (out-degree, DAG in-degree): one 8-byte gather
      else dq[u] = make_int2((int)(g.rowptr[ss[u] + 1] - g.rowptr[ss[u]]), g.indeg ? g.indeg[ss[u]] : 0);
    }
    int32_t wlo[PLAN_UNROLL], whi[PLAN_UNROLL];
#pragma unroll
    for (int u = 0; u < PLAN_UNROLL; ++u) {
      const int64_t e = eb + 32 * u;
      const int64_t s0 = g.restrict_after ? e + 1 : rbs[u];
      const bool wide = e < e1 && pr[u] != rr[u] && s0 < res[u];  // a row start with a window
      wlo[u] = wide ? g.col[s0] : 0;
      whi[u] = wide ? g.col[res[u] - 1] : -1;
    }
#pragma unroll
    for (int u = 0; u < PLAN_UNROLL; ++u) {
      const int64_t e = eb + 32 * u;
      if (e >= e1) break;
      const int64_t rb = rbs[u], re = res[u];
      const int64_t a0 = g.restrict_after ? e + 1 : rb;
      const float da = (float)(re - a0);
      const float db = (float)dq[u].x, ins = (float)dq[u].y;  // target's out-degree and DAG in-degree
      sda += da;
      sdb += db;
      const float mn = fminf(da, db), mx = fmaxf(da, db);
      smin += mn;
      smax += mx;
      const float lr = flog2p1(da) - flog2p1(db);
      salr += fabsf(lr);
      sin += ins;  // how many edges share this target's list
      const int bin = mn < 2.f ? 0 : mn < 8.f ? 1 : mn < 32.f ? 2 : mn < 128.f ? 3 : mn < 512.f ? 4 : 5;
#pragma unroll
      for (int k = 0; k < 6; ++k) bins[k] += (bin == k) ? 1.f : 0.f;
      work += (unsigned long long)(da + db);
      alg += 4ULL * (unsigned long long)((re - rb) + (int64_t)db) + 4ULL;
      if (pr[u] != rr[u]) {  // the edge starts its row in the tile (pr = -1 for the tile's first edge)
        ++nrows;
        maxdr = max(maxdr, (long long)(re - rb));
        maxwin = max(maxwin, (long long)whi[u] - (long long)wlo[u] + 1);
      }
    }
  }
  sda = warp_sum(sda); sdb = warp_sum(sdb); smin = warp_sum(smin); smax = warp_sum(smax);
  salr = warp_sum(salr); sin = warp_sum(sin);
#pragma unroll
  for (int k = 0; k < 6; ++k) bins[k] = warp_sum(bins[k]);
  work = warp_sum(work);
  alg = warp_sum(alg);
  nrows = warp_sum(nrows);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    maxdr = max(maxdr, __shfl_xor_sync(TC_FULL_MASK, maxdr, o));
    maxwin = max(maxwin, __shfl_xor_sync(TC_FULL_MASK, maxwin, o));
  }
  const float ne = (float)(e1 - e0);
  PlanStats st;
  st.mean_da = sda / ne; st.mean_db = sdb / ne; st.mean_min = smin / ne; st.mean_max = smax / ne;
  st.mean_in = sin / ne; st.alr = salr / ne;
  st.nrows = (float)nrows; st.maxdr = (float)maxdr; st.maxwin = (float)maxwin; st.frac = ne / (float)TILE_EDGES;
  float f[TC_MLP_FEATURES];
  f[0] = flog2p1(st.mean_da) / 16.f;
  f[1] = flog2p1(st.mean_db) / 16.f;
  f[2] = flog2p1(st.mean_in) / 24.f;
  f[3] = st.alr / 16.f;
  f[4] = flog2p1(st.mean_min) / 16.f;
  f[5] = flog2p1(st.mean_max) / 16.f;
  f[6] = flog2p1(st.nrows) / 12.f;
  f[7] = flog2p1(st.maxdr) / 16.f;
#pragma unroll
  for (int k = 0; k < 6; ++k) f[8 + k] = bins[k] / ne;
  f[14] = flog2p1(st.maxwin) / 24.f;
  f[15] = flog2p1((float)g.m) / 32.f;  // graph size: how much of it the L2 can hold
  int arm;
  if (selector == TC_SELECT_FORCE) arm = force_arm;
  else if (selector == TC_SELECT_LEARNED) {
    // The fixed rule keeps the PULL decision: a PULL tile's cost depends on
    // how many of its targets' in-edges other PULL tiles share (the table
    // build is spread over them), which per-tile costs profiled one arm at a
    // time cannot show.  The cost model picks among the per-edge arms for
    // every other tile.
    const int fx = __shfl_sync(TC_FULL_MASK, fixed_select(st), 0);
    arm = fx == TC_ARM_PULL ? TC_ARM_PULL : mlp_select(s_w, f, lane, TC_ARM_PULL, fx, margin);
  } else {
    arm = fixed_select(st);
  }
  arm = __shfl_sync(TC_FULL_MASK, arm, 0);
  if (lane < TC_MLP_FEATURES) feats[t * TC_MLP_FEATURES + lane] = f[lane];
  if (arm == TC_ARM_PULL) {
    const int64_t kb = pk.block_base(t), lb = pk.low_base(t);
    for (int64_t e = e0 + lane; e < e1; e += 32) atomicAdd(pull_cnt + pk.key_in(kb, lb, g.col[e]), 1u);
  }
  if (lane == 0) {
    arm_out[t] = arm;
    const unsigned long long W40 = (1ULL << 40) - 1;
    qkeys[t] = ((unsigned long long)arm << 40) | (W40 - min(work, W40));
    qvals[t] = (uint32_t)t;
    tile_bytes[t] = alg;
  }
}

// Algorithmic bytes of every arm's tiles (block a sums queue a).
__global__ void arm_bytes_kernel(const uint32_t *__restrict__ qtiles, const int64_t *__restrict__ qoff,
                                 const unsigned long long *__restrict__ tile_bytes,
                                 unsigned long long *__restrict__ out) {
  __shared__ unsigned long long part[8];
  const int a = blockIdx.x;
  unsigned long long s = 0;
  for (int64_t i = qoff[a] + threadIdx.x; i < qoff[a + 1]; i += blockDim.x) s += tile_bytes[qtiles[i]];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
    out[a] = t;
  }
}

__global__ void qoff_kernel(const uint64_t *__restrict__ keys, int64_t T, int64_t *__restrict__ qoff) {
  const int k = threadIdx.x;
  if (k > TC_NUM_ARMS) return;
  int64_t lo = 0, hi = T;  // first index with arm >= k
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if ((int64_t)(keys[mid] >> 40) < k) lo = mid + 1; else hi = mid;
  }
  qoff[k] = lo;
}

// ---- shared pieces of the arm kernels -----------------------------------------

struct EdgeLists {
  const int32_t *a;  // remaining out-list of the row
  const int32_t *b;  // out-list of the column vertex
  int na, nb;
};

__device__ __forceinline__ EdgeLists edge_lists(const DevDag &g, int64_t e, int32_t &s_out) {
  const int32_t r = g.src[e], s = g.col[e];
  s_out = s;
  const int64_t rb = g.rowptr[r], re = g.rowptr[r + 1];
  const int64_t a0 = g.restrict_after ? e + 1 : rb;
  const int64_t sb = g.rowptr[s], se = g.rowptr[s + 1];
  EdgeLists L;
  L.a = g.col + a0;
  L.na = (int)(re - a0);
  L.b = g.col + sb;
  L.nb = (int)(se - sb);
  return L;
}

__device__ __forceinline__ void put_edge_count(const DevDag &g, uint32_t *out, int64_t e, uint32_t c) {
  if (out) out[g.perm ? (int64_t)g.perm[e] : e] = c;
}

// Pull the next tile of this arm's queue (block-uniform result).
__device__ __forceinline__ int64_t next_tile(const uint32_t *__restrict__ qtiles, int64_t qb, int64_t qn,
                                             unsigned *head, int64_t *s_tile) {
  if (threadIdx.x == 0) {
    const unsigned it = atomicAdd(head, 1u);
    *s_tile = (int64_t)it < qn ? (int64_t)qtiles[qb + it] : -1;
  }
  __syncthreads();
  const int64_t t = *s_tile;
  __syncthreads();
  return t;
}

// The group arms (BSEARCH_G, MERGE_G, GALLOP_G, MPATH_G) take their tiles in
// GROUP_SUBS pieces (512 edges each), so an arm that gets a few heavy tiles
// spreads them over several blocks instead of leaving one block to finish a
// whole tile while the rest of the GPU waits.
#ifndef TC_GROUP_SUBS
#define TC_GROUP_SUBS 8
#endif
constexpr int GROUP_SUBS = TC_GROUP_SUBS;

// Next piece of this arm's queue (block-uniform): its tile and edge range.
__device__ __forceinline__ bool next_sub_tile(const uint32_t *__restrict__ qtiles, int64_t qb, int64_t qn,
                                              unsigned *head, int64_t *s_item, int64_t m, int64_t *tile,
                                              int64_t *e0, int64_t *e1) {
  if (threadIdx.x == 0) {
    const unsigned it = atomicAdd(head, 1u);
    *s_item = (int64_t)it < qn * GROUP_SUBS
                  ? (int64_t)qtiles[qb + it / GROUP_SUBS] * GROUP_SUBS + (int64_t)(it % GROUP_SUBS)
                  : -1;
  }
  __syncthreads();
  const int64_t item = *s_item;
  __syncthreads();
  if (item < 0) return false;
  constexpr int64_t SUB = TILE_EDGES / GROUP_SUBS;
  *tile = item / GROUP_SUBS;
  *e0 = *tile * TILE_EDGES + (item % GROUP_SUBS) * SUB;
  *e1 = min(m, *e0 + SUB);
  return true;
}

__device__ __forceinline__ void flush_total(unsigned long long acc, unsigned long long *total) {
  __shared__ unsigned long long s_acc;
  if (threadIdx.x == 0) s_acc = 0;
  __syncthreads();
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(&s_acc, acc);
  __syncthreads();
  if (threadIdx.x == 0 && s_acc) atomicAdd(total, s_acc);
}

// Count of keys of sorted `l` (nl) present in sorted `s` (ns), lanes
// gl, gl+G, ... of a G-lane group; the search window's lower end only moves
// forward because keys grow.
template <int G>
__device__ __forceinline__ uint32_t bsearch_count(const int32_t *__restrict__ l, int nl,
                                                  const int32_t *__restrict__ s, int ns, int gl) {
  uint32_t c = 0;
  int lo = 0;
  for (int i = gl; i < nl; i += G) {
    const int32_t key = __ldg(l + i);
    int hi = ns;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (__ldg(s + mid) < key) lo = mid + 1; else hi = mid;
    }
    if (lo < ns && __ldg(s + lo) == key) ++c;
  }
  return c;
}

// Same count with K independent binary searches in flight per lane: lane gl
// takes keys gl + k*G of each G*K-key batch; the K searches advance in
// lockstep, so their loads issue back to back instead of one dependent chain
// at a time.  Keys grow along a lane, so the next batch starts its searches
// at the last key's lower bound.
template <int G, int K>
__device__ __forceinline__ uint32_t bsearch_count_ilp(const int32_t *__restrict__ l, int nl,
                                                      const int32_t *__restrict__ s, int ns, int gl) {
  uint32_t c = 0;
  int base = 0;
  for (int i0 = gl; i0 < nl; i0 += G * K) {
    int32_t key[K];
    int lo[K], hi[K];
    int last = 0;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int idx = i0 + k * G;
      const bool act = idx < nl;
      key[k] = act ? __ldg(l + idx) : INT32_MAX;
      lo[k] = base;
      hi[k] = act ? ns : base;  // inactive searches are empty
      last = act ? k : last;
    }
    int width = ns - base;
    while (width > 0) {  // ceil(log2(width + 1)) rounds bound every search
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if (lo[k] < hi[k]) {
          const int mid = (lo[k] + hi[k]) >> 1;
          if (__ldg(s + mid) < key[k]) lo[k] = mid + 1; else hi[k] = mid;
        }
      }
      width >>= 1;
    }
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (key[k] != INT32_MAX && lo[k] < ns && __ldg(s + lo[k]) == key[k]) ++c;
    base = lo[last];
  }
  return c;
}

// Warp-wide count with a pivot cache: lane l holds s[l*ns/32] (the whole
// list when ns <= 32), so the first five levels of every search are
// register shuffles; the rest is a binary search inside one 1/32 segment.
// All lanes run the same number of rounds (shuffles need the full warp).
__device__ __forceinline__ uint32_t pivot_search_count(const int32_t *__restrict__ l, int nl,
                                                       const int32_t *__restrict__ s, int ns, int lane) {
  const bool small = ns <= 32;
  const int32_t piv = small ? (lane < ns ? __ldg(s + lane) : INT32_MAX)
                            : __ldg(s + (int)(((long long)lane * ns) >> 5));
  uint32_t c = 0;
  for (int i0 = 0; i0 < nl; i0 += 32) {  // warp-uniform trip count
    const int i = i0 + lane;
    const int32_t key = i < nl ? __ldg(l + i) : INT32_MIN;  // INT32_MIN matches nothing
    // p = largest pivot index with piv[p] <= key, or -1 when key < piv[0]
    int p = -1;
#pragma unroll
    for (int step = 32; step >= 1; step >>= 1) {  // p reaches every value in [-1, 31]
      const int32_t pv = __shfl_sync(TC_FULL_MASK, piv, min(p + step, 31));
      if (p + step <= 31 && pv <= key) p += step;
    }
    const int32_t at_p = __shfl_sync(TC_FULL_MASK, piv, p < 0 ? 0 : p);
    if (i >= nl || p < 0) continue;
    if (small) {  // the pivots are the list itself
      c += (at_p == key) ? 1u : 0u;
      continue;
    }
    // s[p*ns/32] <= key < s[(p+1)*ns/32]: the lower bound lies in that segment
    int lo = (int)(((long long)p * ns) >> 5);
    int hi = (int)(((long long)(p + 1) * ns) >> 5);
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (__ldg(s + mid) < key) lo = mid + 1; else hi = mid;
    }
    if (lo < ns && __ldg(s + lo) == key) ++c;
  }
  return c;
}

template <int G>
__device__ __forceinline__ uint32_t group_sum(uint32_t v, unsigned gmask) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(gmask, v, o, G);
  return v;
}

template <int G>
__device__ __forceinline__ unsigned group_mask(int lane) {
  if (G == 32) return TC_FULL_MASK;
  return ((1u << G) - 1u) << (lane & ~(G - 1));
}

// ---- BSEARCH_G ------------------------------------------------------------------

template <int G>
__global__ void __launch_bounds__(CT_THREADS) bsearch_kernel(DevDag g, const uint32_t *__restrict__ qtiles,
                                                            const int64_t *__restrict__ qoff, int arm,
                                                            unsigned *head, uint32_t *out,
                                                            unsigned long long *total,
                                                            unsigned long long *tile_cycles) {
  __shared__ int64_t s_tile;
  const int64_t qb = qoff[arm], qn = qoff[arm + 1] - qb;
  const int lane = threadIdx.x & 31, gl = threadIdx.x % G, gid = threadIdx.x / G;
  constexpr int NG = CT_THREADS / G;
  const unsigned gm = group_mask<G>(lane);
  unsigned long long acc = 0;
  for (;;) {
    int64_t tile, e0, e1;
    if (!next_sub_tile(qtiles, qb, qn, head, &s_tile, g.m, &tile, &e0, &e1)) break;
    const long long c0 = clock64();
    for (int64_t e = e0 + gid; e < e1; e += NG) {
      int32_t s;
      const EdgeLists L = edge_lists(g, e, s);
      uint32_t c = 0;
      if (L.na > 0 && L.nb > 0) {
        // narrow groups keep 4 searches in flight per lane; a full warp per
        // edge already has 32 in flight and runs them one at a time
        if (G <= 8) {
          if (L.na <= L.nb) c = bsearch_count_ilp<G, 4>(L.a, L.na, L.b, L.nb, gl);
          else c = bsearch_count_ilp<G, 4>(L.b, L.nb, L.a, L.na, gl);
        } else if (G == 32) {
          if (L.na <= L.nb) c = pivot_search_count(L.a, L.na, L.b, L.nb, lane);
          else c = pivot_search_count(L.b, L.nb, L.a, L.na, lane);
        } else {
          if (L.na <= L.nb) c = bsearch_count<G>(L.a, L.na, L.b, L.nb, gl);
          else c = bsearch_count<G>(L.b, L.nb, L.a, L.na, gl);
        }
      }
      c = group_sum<G>(c, gm);
      if (gl == 0) {
        put_edge_count(g, out, e, c);
        acc += c;
      }
    }
    if (tile_cycles) {
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(&tile_cycles[tile], (unsigned long long)(clock64() - c0));
    }
  }
  flush_total(acc, total);
}

// ---- BSEARCH_32 with the search list staged by bulk copies ----------------------
//
// One warp per edge, as in the reference's warp_intersect (graph_gpu.h:228-252):
// lanes take keys of the shorter list and binary-search them in the longer
// one.  Here the longer list is first copied into the warp's shared memory by
// one bulk asynchronous copy (cp.async.bulk, the TMA unit's non-tensor form)
// completing an mbarrier, so every search step reads shared memory instead of
// making a dependent trip to L2; the copy of the warp's next edge is issued
// before the current edge is searched, so it overlaps that search.  The copy
// covers the 16-byte blocks that hold the list (at most 3 entries either
// side; an aligned block holding a list entry lies in that entry's memory
// page), and the search skips to the list's offset in the buffer.  Lists
// longer than a buffer are searched in place (pivot search).  A wait that
// gives up (it should never) sets VF_TIMEOUT and the warp counts its
// remaining edges in place, after waiting (bounded) for its copies in flight.
// 1: BSEARCH_32 searches the longer list in place (pivot search), for
// measuring the staged version against it.
#ifndef TC_BS32_PIVOT
#define TC_BS32_PIVOT 0
#endif
constexpr int BT_STAGE = 512;         // entries per staging buffer (static shared memory stays under 48 KB)
constexpr int BT_WARPS = CT_THREADS / 32;
constexpr uint32_t BT_WAIT_LIMIT = 1u << 22;

struct BtEdge {
  const int32_t *keys;   // shorter list (global)
  const int32_t *list;   // longer list (global)
  int nk, nl;
  int off;               // list's first entry in the staging buffer (staged only)
  bool staged;
};

// Issues the copy of edge e's longer list into buf (lane 0), or marks it to be
// searched in place.
__device__ __forceinline__ BtEdge bt_issue(const DevDag &g, int64_t e, int32_t *buf, uint64_t *bar, bool stage_ok,
                                           int lane) {
  int32_t s;
  const EdgeLists L = edge_lists(g, e, s);
  BtEdge b;
  const bool a_short = L.na <= L.nb;
  b.keys = a_short ? L.a : L.b;
  b.nk = a_short ? L.na : L.nb;
  b.list = a_short ? L.b : L.a;
  b.nl = a_short ? L.nb : L.na;
  b.off = 0;
  b.staged = false;
  // staging pays when the searches touch more of the list than the copy
  // moves: about nk * log2(nl) probes of a 32-byte sector each against 4*nl
  // bytes copied
  if (!stage_ok || b.nk <= 0 || b.nl <= 32 || b.nl > BT_STAGE ||
      8 * b.nk * (32 - __clz(b.nl)) < b.nl)
    return b;
  const uintptr_t a0 = reinterpret_cast<uintptr_t>(b.list);
  const uintptr_t lo = a0 & ~(uintptr_t)15, hi = (a0 + 4 * (uintptr_t)b.nl + 15) & ~(uintptr_t)15;
  b.off = (int)((a0 - lo) >> 2);
  b.staged = true;
  if (lane == 0) {
    fence_proxy_async_smem();  // this warp's earlier reads of buf come first
    mbar_arrive_expect_tx(bar, (uint32_t)(hi - lo));
    bulk_copy_g2s(buf, reinterpret_cast<const void *>(lo), (uint32_t)(hi - lo), bar);
  }
  return b;
}

__device__ __forceinline__ uint32_t bt_count_staged(const BtEdge &b, const int32_t *buf, int lane) {
  const int32_t *S = buf + b.off;
  uint32_t c = 0;
  int lo = 0;
  for (int i = lane; i < b.nk; i += 32) {  // keys ascend, so each lane's lower bound only moves up
    const int32_t key = __ldg(b.keys + i);
    int hi = b.nl;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (S[mid] < key) lo = mid + 1; else hi = mid;
    }
    if (lo < b.nl && S[lo] == key) ++c;
  }
  return c;
}

__global__ void __launch_bounds__(CT_THREADS) bsearch_tma_kernel(DevDag g, const uint32_t *__restrict__ qtiles,
                                                                const int64_t *__restrict__ qoff, int arm,
                                                                unsigned *head, uint32_t *out,
                                                                unsigned long long *total,
                                                                unsigned long long *tile_cycles) {
  __shared__ __align__(16) int32_t stage[BT_WARPS][2][BT_STAGE + 8];
  __shared__ __align__(8) uint64_t bar[BT_WARPS][2];
  __shared__ int64_t s_tile;
  const int64_t qb = qoff[arm], qn = qoff[arm + 1] - qb;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    mbar_init(&bar[w][0], 1);
    mbar_init(&bar[w][1], 1);
    fence_mbar_init();
  }
  __syncwarp();
  uint32_t parity[2] = {0u, 0u};  // parity of the next phase of each buffer's barrier
  bool stage_ok = true;           // false after a wait gave up: this warp stops staging
  bool pending[2] = {false, false};
  unsigned long long acc = 0;
  for (;;) {
    int64_t tile, e0, e1;
    if (!next_sub_tile(qtiles, qb, qn, head, &s_tile, g.m, &tile, &e0, &e1)) break;
    const long long c0 = clock64();
    int cur = 0;
    int64_t e = e0 + w;
    BtEdge b = {};
    if (e < e1) {
      b = bt_issue(g, e, stage[w][cur], &bar[w][cur], stage_ok, lane);
      pending[cur] = b.staged;
    }
    for (; e < e1; e += BT_WARPS) {
      BtEdge nb = {};
      const int64_t en = e + BT_WARPS;
      if (en < e1) {  // the next edge's copy overlaps this edge's search
        nb = bt_issue(g, en, stage[w][cur ^ 1], &bar[w][cur ^ 1], stage_ok, lane);
        pending[cur ^ 1] = nb.staged;
      }
      uint32_t c = 0;
      bool in_place = !b.staged;
      if (b.staged) {
        const bool ok = mbar_wait_bounded(&bar[w][cur], parity[cur], BT_WAIT_LIMIT);
        if (__all_sync(TC_FULL_MASK, ok)) {
          parity[cur] ^= 1u;
          pending[cur] = false;
        } else {  // give up staging; count in place
          if (lane == 0 && g.flags) atomicOr(g.flags, (unsigned)VF_TIMEOUT);
          stage_ok = false;
          in_place = true;
        }
      }
      if (!in_place) c = bt_count_staged(b, stage[w][cur], lane);
      else if (b.nk > 0 && b.nl > 0) c = pivot_search_count(b.keys, b.nk, b.list, b.nl, lane);
      c = warp_sum(c);
      if (lane == 0) {
        put_edge_count(g, out, e, c);
        acc += c;
      }
      __syncwarp();  // every lane is done with this buffer before it takes a new copy
      cur ^= 1;
      b = nb;
    }
    if (tile_cycles) {
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(&tile_cycles[tile], (unsigned long long)(clock64() - c0));
    }
  }
  // a copy left in flight by a wait that gave up lands before the block exits
  for (int k = 0; k < 2; ++k)
    if (pending[k]) (void)mbar_wait_bounded(&bar[w][k], parity[k], BT_WAIT_LIMIT);
  flush_total(acc, total);
}

// ---- MERGE_G ---------------------------------------------------------------------

template <int G>
__device__ __forceinline__ uint32_t merge_count(const int32_t *__restrict__ A, int na, const int32_t *__restrict__ B,
                                                int nb, int gl, unsigned gm) {
  uint32_t c = 0;
  int i = 0, j = 0;
  while (i < na && j < nb) {
    const int32_t av = (i + gl < na) ? __ldg(A + i + gl) : INT32_MAX;
    const int32_t bv = (j + gl < nb) ? __ldg(B + j + gl) : INT32_MAX;
    const int32_t alast = __shfl_sync(gm, av, min(G - 1, na - i - 1), G);
    const int32_t blast = __shfl_sync(gm, bv, min(G - 1, nb - j - 1), G);
    int pos = 0;
#pragma unroll
    for (int step = G / 2; step > 0; step >>= 1) {
      const int32_t probe = __shfl_sync(gm, bv, pos + step - 1, G);
      if (probe < av) pos += step;
    }
    const int32_t hit = __shfl_sync(gm, bv, pos, G);
    if (av != INT32_MAX && hit == av) ++c;
    if (alast <= blast) i += G;
    if (blast <= alast) j += G;
  }
  return c;
}

template <int G>
__global__ void __launch_bounds__(CT_THREADS) merge_kernel(DevDag g, const uint32_t *__restrict__ qtiles,
                                                          const int64_t *__restrict__ qoff, int arm, unsigned *head,
                                                          uint32_t *out, unsigned long long *total,
                                                          unsigned long long *tile_cycles) {
  __shared__ int64_t s_tile;
  const int64_t qb = qoff[arm], qn = qoff[arm + 1] - qb;
  const int lane = threadIdx.x & 31, gl = threadIdx.x % G, gid = threadIdx.x / G;
  constexpr int NG = CT_THREADS / G;
  const unsigned gm = group_mask<G>(lane);
  unsigned long long acc = 0;
  for (;;) {
    int64_t tile, e0, e1;
    if (!next_sub_tile(qtiles, qb, qn, head, &s_tile, g.m, &tile, &e0, &e1)) break;
    const long long c0 = clock64();
    for (int64_t e = e0 + gid; e < e1; e += NG) {
      int32_t s;
      const EdgeLists L = edge_lists(g, e, s);
      uint32_t c = 0;
      if (L.na > 0 && L.nb > 0) c = merge_count<G>(L.a, L.na, L.b, L.nb, gl, gm);
      c = group_sum<G>(c, gm);
      if (gl == 0) {
        put_edge_count(g, out, e, c);
        acc += c;
      }
    }
    if (tile_cycles) {
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(&tile_cycles[tile], (unsigned long long)(clock64() - c0));
    }
  }
  flush_total(acc, total);
}

// ---- GALLOP_G ---------------------------------------------------------------------
//
// Lane gl of a G-lane group takes the contiguous run [gl*nl/G, (gl+1)*nl/G)
// of the shorter list and walks it through the longer list with galloping
// (exponential then binary) searches, each starting where the previous key
// landed: O(nl/G * log(ns/nl)) steps, mostly within the cache lines the
// previous key touched.

// First p in [pos, n) with L[p] >= key (n if none).
__device__ __forceinline__ int gallop_lb(const int32_t *__restrict__ L, int n, int pos, int32_t key) {
  if (pos >= n || __ldg(L + pos) >= key) return pos;
  int lo = pos, step = 1, hi;
  for (;;) {  // invariant: L[lo] < key
    hi = lo + step;
    if (hi >= n) { hi = n; break; }
    if (__ldg(L + hi) >= key) break;
    lo = hi;
    step <<= 1;
  }
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(L + mid) < key) lo = mid; else hi = mid;
  }
  return hi;
}

template <int G>
__device__ __forceinline__ uint32_t gallop_count(const int32_t *__restrict__ s, int ns, const int32_t *__restrict__ l,
                                                 int nl, int gl) {
  const int k0 = (int)(((long long)gl * ns) / G), k1 = (int)(((long long)(gl + 1) * ns) / G);
  uint32_t c = 0;
  if (k0 >= k1) return 0;
  int pos = 0;
  // the run's first key: plain binary search over the whole longer list
  {
    const int32_t key = __ldg(s + k0);
    int lo = 0, hi = nl;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (__ldg(l + mid) < key) lo = mid + 1; else hi = mid;
    }
    pos = lo;
    if (pos < nl && __ldg(l + pos) == key) { ++c; ++pos; }
  }
  for (int k = k0 + 1; k < k1 && pos < nl; ++k) {
    const int32_t key = __ldg(s + k);
    pos = gallop_lb(l, nl, pos, key);
    if (pos < nl && __ldg(l + pos) == key) { ++c; ++pos; }
  }
  return c;
}

template <int G>
__global__ void __launch_bounds__(CT_THREADS) gallop_kernel(DevDag g, const uint32_t *__restrict__ qtiles,
                                                           const int64_t *__restrict__ qoff, int arm, unsigned *head,
                                                           uint32_t *out, unsigned long long *total,
                                                           unsigned long long *tile_cycles) {
  __shared__ int64_t s_tile;
  const int64_t qb = qoff[arm], qn = qoff[arm + 1] - qb;
  const int lane = threadIdx.x & 31, gl = threadIdx.x % G, gid = threadIdx.x / G;
  constexpr int NG = CT_THREADS / G;
  const unsigned gm = group_mask<G>(lane);
  unsigned long long acc = 0;
  for (;;) {
    int64_t tile, e0, e1;
    if (!next_sub_tile(qtiles, qb, qn, head, &s_tile, g.m, &tile, &e0, &e1)) break;
    const long long c0 = clock64();
    for (int64_t e = e0 + gid; e < e1; e += NG) {
      int32_t s;
      const EdgeLists L = edge_lists(g, e, s);
      uint32_t c = 0;
      if (L.na > 0 && L.nb > 0) {
        if (L.na <= L.nb) c = gallop_count<G>(L.a, L.na, L.b, L.nb, gl);
        else c = gallop_count<G>(L.b, L.nb, L.a, L.na, gl);
      }
      c = group_sum<G>(c, gm);
      if (gl == 0) {
        put_edge_count(g, out, e, c);
        acc += c;
      }
    }
    if (tile_cycles) {
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(&tile_cycles[tile], (unsigned long long)(clock64() - c0));
    }
  }
  flush_total(acc, total);
}

// ---- MPATH_G -----------------------------------------------------------------------
//
// Merge-path intersection: the merged order of A and B (A first on ties) is
// cut into G equal segments; lane gl finds its cut (i, d - i) by a binary
// search on its diagonal d, then merges its segment sequentially and counts a
// match when a B element equals the most recent A element (which may lie
// just before the segment).  Strictly increasing lists make every common
// element counted exactly once.

// Number of A elements among the first d merged elements.
__device__ __forceinline__ int mpath_split(const int32_t *__restrict__ A, int na, const int32_t *__restrict__ B, int nb,
                                           int d) {
  int lo = max(0, d - nb), hi = min(d, na);
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(A + mid) <= __ldg(B + d - mid - 1)) lo = mid + 1; else hi = mid;
  }
  return lo;
}

template <int G>
__device__ __forceinline__ uint32_t mpath_count(const int32_t *__restrict__ A, int na, const int32_t *__restrict__ B,
                                                int nb, int gl, unsigned gm) {
  const int total = na + nb;
  const int d0 = (int)(((long long)gl * total) / G);
  const int i0 = mpath_split(A, na, B, nb, d0);
  int i1 = __shfl_down_sync(gm, i0, 1, G);
  int d1 = __shfl_down_sync(gm, d0, 1, G);
  if (gl == G - 1) { i1 = na; d1 = total; }
  const int j0 = d0 - i0, j1 = d1 - i1;
  int i = i0, j = j0;
  int32_t last_a = i0 > 0 ? __ldg(A + i0 - 1) : INT32_MIN;
  uint32_t c = 0;
  for (int step = d0; step < d1; ++step) {
    const int32_t av = i < i1 ? __ldg(A + i) : INT32_MAX;
    const int32_t bv = j < j1 ? __ldg(B + j) : INT32_MAX;
    const bool take_a = (i < i1) && (j >= j1 || av <= bv);
    if (take_a) {
      last_a = av;
      ++i;
    } else {
      c += (bv == last_a) ? 1u : 0u;
      ++j;
    }
  }
  return c;
}

template <int G>
__global__ void __launch_bounds__(CT_THREADS) mpath_kernel(DevDag g, const uint32_t *__restrict__ qtiles,
                                                          const int64_t *__restrict__ qoff, int arm, unsigned *head,
                                                          uint32_t *out, unsigned long long *total,
                                                          unsigned long long *tile_cycles) {
  __shared__ int64_t s_tile;
  const int64_t qb = qoff[arm], qn = qoff[arm + 1] - qb;
  const int lane = threadIdx.x & 31, gl = threadIdx.x % G, gid = threadIdx.x / G;
  constexpr int NG = CT_THREADS / G;
  const unsigned gm = group_mask<G>(lane);
  unsigned long long acc = 0;
  for (;;) {
    int64_t tile, e0, e1;
    if (!next_sub_tile(qtiles, qb, qn, head, &s_tile, g.m, &tile, &e0, &e1)) break;
    const long long c0 = clock64();
    for (int64_t e = e0 + gid; e < e1; e += NG) {
      int32_t s;
      const EdgeLists L = edge_lists(g, e, s);
      uint32_t c = 0;
      if (L.na > 0 && L.nb > 0) c = mpath_count<G>(L.a, L.na, L.b, L.nb, gl, gm);
      c = group_sum<G>(c, gm);
      if (gl == 0) {
        put_edge_count(g, out, e, c);
        acc += c;
      }
    }
    if (tile_cycles) {
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(&tile_cycles[tile], (unsigned long long)(clock64() - c0));
    }
  }
  flush_total(acc, total);
}

// ---- FLAT (warp-level, flattened binary searches) -----------------------------------
//
// A warp owns a 512-edge sub-tile and takes 32 edges at a time: lane i loads
// edge i's lists (the shorter one is the lookup list) and the warp walks the
// concatenation of the 32 lookup lists, lane p searching element p of it in
// its edge's longer list, FL_K searches in flight per lane.  Short and long
// lookups share the lanes evenly; a lane's successive keys in one edge grow,
// so each search starts at the lane's previous lower bound in that edge.

constexpr int FL_THREADS = 256;
constexpr int FL_WARPS = FL_THREADS / 32;
constexpr int FL_K = 4;
constexpr int FL_SUB = TILE_EDGES / 8;  // edges per warp work item

__global__ void __launch_bounds__(FL_THREADS) flat_kernel(DevDag g, const uint32_t *__restrict__ qtiles,
                                                         const int64_t *__restrict__ qoff, int arm, unsigned *head,
                                                         uint32_t *out, unsigned long long *total,
                                                         unsigned long long *tile_cycles) {
  __shared__ int32_t s_incl[FL_WARPS][32];
  __shared__ long long s_lbase[FL_WARPS][32];  // lookup list start minus its first flattened index
  __shared__ long long s_sbase[FL_WARPS][32];  // search list start
  __shared__ int32_t s_slen[FL_WARPS][32];
  __shared__ uint32_t s_hits[FL_WARPS][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t qb = qoff[arm], qn = qoff[arm + 1] - qb;
  const int64_t items = qn * (TILE_EDGES / FL_SUB);
  unsigned long long acc = 0;
  for (;;) {
    unsigned it = 0;
    if (lane == 0) it = atomicAdd(head, 1u);
    it = __shfl_sync(TC_FULL_MASK, it, 0);
    if ((int64_t)it >= items) break;
    const int64_t tile = qtiles[qb + it / (TILE_EDGES / FL_SUB)];
    const int64_t e0 = tile * TILE_EDGES + (int64_t)(it % (TILE_EDGES / FL_SUB)) * FL_SUB;
    const int64_t e1 = min(g.m, e0 + FL_SUB);
    const long long c0 = clock64();
    for (int64_t eb = e0; eb < e1; eb += 32) {
      const int64_t ei = eb + lane;
      int nl = 0, ns = 0;
      long long lb = 0, sb = 0;
      if (ei < e1) {
        int32_t s;
        const EdgeLists L = edge_lists(g, ei, s);
        if (L.na > 0 && L.nb > 0) {
          const bool a_short = L.na <= L.nb;
          nl = a_short ? L.na : L.nb;
          ns = a_short ? L.nb : L.na;
          lb = (a_short ? L.a : L.b) - g.col;
          sb = (a_short ? L.b : L.a) - g.col;
        }
      }
      int incl = nl;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(TC_FULL_MASK, incl, o);
        if (lane >= o) incl += y;
      }
      const int P = __shfl_sync(TC_FULL_MASK, incl, 31);
      s_incl[w][lane] = incl;
      s_lbase[w][lane] = lb - (long long)(incl - nl);
      s_sbase[w][lane] = sb;
      s_slen[w][lane] = ns;
      s_hits[w][lane] = 0u;
      __syncwarp();
      int cur = 0;          // edge of the lane's current key
      int lo_edge = -1;     // edge whose lower bound prev_lo is (last finished search)
      int prev_lo = 0;
      for (int p0 = lane; p0 < P; p0 += 32 * FL_K) {
        int32_t key[FL_K];
        int lo[FL_K], hi[FL_K], ed[FL_K];
        long long sbase[FL_K];
        int width = 0;
#pragma unroll
        for (int k = 0; k < FL_K; ++k) {
          const int p = p0 + 32 * k;
          ed[k] = -1;
          lo[k] = hi[k] = 0;
          key[k] = 0;
          sbase[k] = 0;
          if (p < P) {
            while (s_incl[w][cur] <= p) ++cur;
            ed[k] = cur;
            key[k] = __ldg(g.col + s_lbase[w][cur] + p);
            sbase[k] = s_sbase[w][cur];
            hi[k] = s_slen[w][cur];
            lo[k] = (cur == lo_edge) ? prev_lo : 0;
            width = max(width, hi[k] - lo[k]);
          }
        }
        while (width > 0) {
#pragma unroll
          for (int k = 0; k < FL_K; ++k) {
            if (lo[k] < hi[k]) {
              const int mid = (lo[k] + hi[k]) >> 1;
              if (__ldg(g.col + sbase[k] + mid) < key[k]) lo[k] = mid + 1; else hi[k] = mid;
            }
          }
          width >>= 1;
        }
#pragma unroll
        for (int k = 0; k < FL_K; ++k) {
          if (ed[k] >= 0) {
            if (lo[k] < s_slen[w][ed[k]] && __ldg(g.col + sbase[k] + lo[k]) == key[k]) atomicAdd(&s_hits[w][ed[k]], 1u);
            prev_lo = lo[k];  // keys grow along the lane: a valid start for its next key in this edge
            lo_edge = ed[k];
          }
        }
      }
      __syncwarp();
      if (ei < e1) {
        const uint32_t c = s_hits[w][lane];
        put_edge_count(g, out, ei, c);
        acc += c;
      }
      __syncwarp();
    }
    if (tile_cycles && lane == 0) atomicAdd(&tile_cycles[tile], (unsigned long long)(clock64() - c0));
  }
  flush_total(acc, total);
}

// ---- HASH (warp-level, row-staged) ---------------------------------------------------
//
// A warp owns a 512-edge sub-tile pulled from the arm's queue.  For every
// row segment in it, the warp hashes the row's remaining out-list (elements
// after the segment's first edge: earlier ones are <= that edge's target
// and cannot meet its out-list) into its own shared-memory table
// (multiplicative hashing, linear probing, load <= 1/2), then streams the
// out-lists of up to 32 of the segment's edges at once as one flattened
// sequence: lane p of a pass reads element p of the concatenation, so short
// lists do not idle lanes and each list is read with coalesced loads.  Hits
// are rare (they are triangles) and go to a shared per-edge counter.

constexpr int HT_THREADS = 256;
constexpr int HT_WARPS = HT_THREADS / 32;
constexpr int HT_SLOTS = 1024;               // per warp: rows with <= 512 remaining entries
constexpr int SUB_EDGES = TILE_EDGES / 8;    // warp work item
constexpr int32_t HT_EMPTY = -1;

__device__ __forceinline__ uint32_t hslot(int32_t x, int bits) {
  return ((uint32_t)x * 0x9E3779B1u) >> (32 - bits);
}

__global__ void __launch_bounds__(HT_THREADS) hash_kernel(DevDag g, const uint32_t *__restrict__ qtiles,
                                                         const int64_t *__restrict__ qoff, int arm, unsigned *head,
                                                         uint32_t *out, unsigned long long *total,
                                                         unsigned long long *tile_cycles) {
  __shared__ int32_t tab[HT_WARPS][HT_SLOTS];
  __shared__ int32_t s_incl[HT_WARPS][32];
  __shared__ long long s_base[HT_WARPS][32];  // list start minus the list's first flattened index
  __shared__ uint32_t s_hits[HT_WARPS][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t *T = tab[w];
  const int64_t qb = qoff[arm], qn = qoff[arm + 1] - qb;
  const int64_t items = qn * (TILE_EDGES / SUB_EDGES);
  unsigned long long acc = 0;
  for (;;) {
    unsigned it = 0;
    if (lane == 0) it = atomicAdd(head, 1u);
    it = __shfl_sync(TC_FULL_MASK, it, 0);
    if ((int64_t)it >= items) break;
    const int64_t tile = qtiles[qb + it / (TILE_EDGES / SUB_EDGES)];
    const int64_t e0 = tile * TILE_EDGES + (int64_t)(it % (TILE_EDGES / SUB_EDGES)) * SUB_EDGES;
    const int64_t e1 = min(g.m, e0 + SUB_EDGES);
    const long long c0 = clock64();
    for (int64_t e = e0; e < e1;) {
      const int32_t r = g.src[e];
      const int64_t rb = g.rowptr[r], re = g.rowptr[r + 1];
      const int64_t se = min(e1, re);
      const int64_t a0 = g.restrict_after ? e + 1 : rb;
      const int na = (int)(re - a0);
      if (na <= 0) {  // nothing after the segment start can be shared
        for (int64_t k = e + lane; k < se; k += 32) put_edge_count(g, out, k, 0u);
        e = se;
        continue;
      }
      if (na > HT_SLOTS / 2) {  // row too long for the warp table: binary search per edge
        for (int64_t k = e; k < se; ++k) {
          int32_t s;
          const EdgeLists L = edge_lists(g, k, s);
          uint32_t c = 0;
          if (L.na > 0 && L.nb > 0) {
            if (L.na <= L.nb) c = bsearch_count<32>(L.a, L.na, L.b, L.nb, lane);
            else c = bsearch_count<32>(L.b, L.nb, L.a, L.na, lane);
          }
          c = warp_sum(c);
          if (lane == 0) {
            put_edge_count(g, out, k, c);
            acc += c;
          }
        }
        e = se;
        continue;
      }
      int bits = 5;
      while ((1 << bits) < 2 * na) ++bits;
      const uint32_t mask = (1u << bits) - 1u;
      for (int k = lane; k < (1 << bits); k += 32) T[k] = HT_EMPTY;
      __syncwarp();
      for (int k = lane; k < na; k += 32) {
        const int32_t x = __ldg(g.col + a0 + k);
        uint32_t sl = hslot(x, bits);
        while (atomicCAS(&T[sl], HT_EMPTY, x) != HT_EMPTY) sl = (sl + 1) & mask;
      }
      const int32_t amax = __ldg(g.col + re - 1);
      __syncwarp();
      for (int64_t eb = e; eb < se; eb += 32) {
        const int64_t ei = eb + lane;
        int nb = 0;
        long long bst = 0;
        if (ei < se) {
          const int32_t s = g.col[ei];
          bst = g.rowptr[s];
          nb = (int)(g.rowptr[s + 1] - bst);
        }
        int incl = nb;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(TC_FULL_MASK, incl, o);
          if (lane >= o) incl += y;
        }
        const int P = __shfl_sync(TC_FULL_MASK, incl, 31);
        s_incl[w][lane] = incl;
        s_base[w][lane] = bst - (long long)(incl - nb);
        s_hits[w][lane] = 0u;
        __syncwarp();
        int i = 0;
        int cur_end = s_incl[w][0];
        long long cur_base = s_base[w][0];
        for (int p = lane; p < P; p += 32) {
          if (p >= cur_end) {
            do { ++i; } while (s_incl[w][i] <= p);
            cur_end = s_incl[w][i];
            cur_base = s_base[w][i];
          }
          const int32_t x = __ldg(g.col + cur_base + p);
          if (x <= amax) {
            uint32_t sl = hslot(x, bits);
            for (;;) {
              const int32_t v = T[sl];
              if (v == x) { atomicAdd(&s_hits[w][i], 1u); break; }
              if (v == HT_EMPTY) break;
              sl = (sl + 1) & mask;
            }
          }
        }
        __syncwarp();
        if (ei < se) {
          const uint32_t c = s_hits[w][lane];
          put_edge_count(g, out, ei, c);
          acc += c;
        }
        __syncwarp();
      }
      e = se;
      __syncwarp();
    }
    if (tile_cycles && lane == 0) atomicAdd(&tile_cycles[tile], (unsigned long long)(clock64() - c0));
  }
  flush_total(acc, total);
}

// ---- BITMAP ------------------------------------------------------------------------

__global__ void __launch_bounds__(BM_THREADS) bitmap_kernel(DevDag g, const uint32_t *__restrict__ qtiles,
                                                           const int64_t *__restrict__ qoff, int arm, unsigned *head,
                                                           uint32_t *out, unsigned long long *total,
                                                           unsigned long long *tile_cycles) {
  extern __shared__ uint32_t bm[];
  __shared__ int64_t s_tile;
  const int64_t qb = qoff[arm], qn = qoff[arm + 1] - qb;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int NW = BM_THREADS / 32;
  unsigned long long acc = 0;
  // The bitmap is cleared once; afterwards every segment unsets exactly the
  // bits it set, so a segment costs its out-degree, not its id window.
  for (int w = threadIdx.x; w < BM_SMEM_BYTES / 4; w += BM_THREADS) bm[w] = 0u;
  __syncthreads();
  for (;;) {
    const int64_t tile = next_tile(qtiles, qb, qn, head, &s_tile);
    if (tile < 0) break;
    const long long c0 = clock64();
    const int64_t e0 = tile * TILE_EDGES, e1 = min(g.m, e0 + TILE_EDGES);
    for (int64_t sb = e0; sb < e1;) {
      const int32_t r = g.src[sb];
      const int64_t rb = g.rowptr[r], re = g.rowptr[r + 1];
      const int64_t se = min(e1, re);
      const int64_t a0 = g.restrict_after ? sb + 1 : rb;
      const int64_t win = (a0 < re) ? (int64_t)g.col[re - 1] - (int64_t)g.col[a0] + 1 : 0;
      if (a0 < re && win <= BM_BITS) {
        const int32_t lo = g.col[a0], hi = g.col[re - 1];
        for (int64_t k = a0 + threadIdx.x; k < re; k += BM_THREADS) {
          const uint32_t x = (uint32_t)(g.col[k] - lo);
          atomicOr(&bm[x >> 5], 1u << (x & 31));
        }
        __syncthreads();
        for (int64_t e = sb + warp; e < se; e += NW) {
          const int32_t s = g.col[e];
          const int32_t *B = g.col + g.rowptr[s];
          const int nb = (int)(g.rowptr[s + 1] - g.rowptr[s]);
          uint32_t c = 0;
          for (int k = lane; k < nb; k += 32) {
            const int32_t w = __ldg(B + k);
            if (w > hi) break;
            if (w >= lo) {
              const uint32_t x = (uint32_t)(w - lo);
              c += (bm[x >> 5] >> (x & 31)) & 1u;
            }
          }
          c = warp_sum(c);
          if (lane == 0) {
            put_edge_count(g, out, e, c);
            acc += c;
          }
        }
        __syncthreads();
        for (int64_t k = a0 + threadIdx.x; k < re; k += BM_THREADS)  // unset this segment's bits
          bm[(uint32_t)(g.col[k] - lo) >> 5] = 0u;
        __syncthreads();
      } else {
        for (int64_t e = sb + warp; e < se; e += NW) {
          int32_t s;
          const EdgeLists L = edge_lists(g, e, s);
          uint32_t c = 0;
          if (L.na > 0 && L.nb > 0) {
            if (L.na <= L.nb) c = pivot_search_count(L.a, L.na, L.b, L.nb, lane);
            else c = pivot_search_count(L.b, L.nb, L.a, L.na, lane);
          }
          c = warp_sum(c);
          if (lane == 0) {
            put_edge_count(g, out, e, c);
            acc += c;
          }
        }
      }
      sb = se;
    }
    if (tile_cycles) {
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(&tile_cycles[tile], (unsigned long long)(clock64() - c0));
    }
  }
  flush_total(acc, total);
}

// Per-vertex and labelled modes, long and wide target lists: the warp's
// lanes binary-search the keys of A in B.  A key found at A[i] counts when
// its label is `label` (lbl set) and adds one to topA[i], the DAG entry of
// A[i] (topA set).
__device__ __forceinline__ uint32_t attr_search_count(const int32_t *__restrict__ A, int na,
                                                      const int32_t *__restrict__ B, int nb, uint32_t *topA,
                                                      const uint8_t *__restrict__ lbl, int label, int lane) {
  uint32_t c = 0;
  for (int i = lane; i < na; i += 32) {
    const int32_t key = __ldg(A + i);
    int lo = 0, hi = nb;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (__ldg(B + mid) < key) lo = mid + 1; else hi = mid;
    }
    if (lo < nb && __ldg(B + lo) == key && (!lbl || lbl[key] == label)) {
      ++c;
      if (topA) atomicAdd(topA + i, 1u);
    }
  }
  return c;
}

// ---- PULL (edges grouped by target) ---------------------------------------------------
//
// The edges of PULL tiles are grouped by target v with one counting sort
// (key histogram, exclusive scan, scatter of (edge, row) records; tiles of
// other arms are skipped whole, so the grouping costs little when no tile
// chose PULL).  A warp takes up to 2048 grouped entries; for each run of
// equal v it loads N+(v) once into its shared-memory bitmap or hash table and
// probes, for every in-edge u->v of the run, the part of N+(u) that can close
// a triangle (the row after v in relabelled order), 32 edges at a time as one
// flattened sequence of 16-byte groups.  Hub targets have thousands of
// in-edges, so one table serves them all and each edge costs its row suffix
// at one shared-memory test per entry, not a search per key.  The order
// inside a group depends on atomics; counts do not.

constexpr int PL_THREADS = 128;
constexpr int PL_WARPS = PL_THREADS / 32;
#ifndef TC_PL_WORDS
#define TC_PL_WORDS 2048
#endif
#ifndef TC_PL_MIN_BLOCKS
#define TC_PL_MIN_BLOCKS 6
#endif
constexpr int PL_WORDS = TC_PL_WORDS;  // per warp: a 65536-id bitmap or a 2048-slot hash table
constexpr int PL_UNROLL = 4;      // table build: list loads in flight per lane
#ifndef TC_PL_GUNROLL
#define TC_PL_GUNROLL 4
#endif
constexpr int PL_GUNROLL = TC_PL_GUNROLL;  // flattened probing: 16-byte loads in flight per lane
constexpr int PL_GROUP_THREADS = 256;
// edges per thread whose atomics are issued together in the scatter (1: at
// R-MAT scale 24, 2 and 4 were 0.3 ms slower; at scale 22 4 was 0.05 ms faster)
#ifndef TC_PL_SCATTER_UNROLL
#define TC_PL_SCATTER_UNROLL 1
#endif
constexpr int PL_SCATTER_UNROLL = TC_PL_SCATTER_UNROLL;
// 1: the scatter streams its column and row reads and its record stores with
// evict-first hints, so the grouping counters (K * 4 bytes) stay in L2
#ifndef TC_PL_SCATTER_STREAM
#define TC_PL_SCATTER_STREAM 1
#endif
constexpr bool PL_SCATTER_STREAM = TC_PL_SCATTER_STREAM != 0;
// Dense edges: an edge u->v whose source is a hub and whose row suffix holds
// more than dense_num / dense_den entries per 32-bit word of v's bitmap
// table (ctx->pull_dense_num / pull_dense_den, 1/1 unless tuned) is counted
// by ANDing u's hub bit row with the table, 32 candidates per word, instead
// of probing the suffix entry by entry.
// Dense edges join two of the top PL_DENSE_HUB ids; their bit rows take
// PL_DENSE_HUB^2 / 8 bytes (512 MB).
constexpr int64_t PL_DENSE_HUB = 65536;
constexpr int PL_DUNROLL = 2;  // dense edges: 16-byte word loads in flight per lane

// One counting sort groups the PULL tiles' edges.  A target among the top
// PL_HUB ids (ids are degree ranks) always fits the bitmap window, since all
// of N+(v) lies in (v, n); those targets, the hubs that most edges point to,
// are grouped per source block (a range of tiles, so a range of rows): key
// block * PL_HUB + (v - hub0).  The blocks' groups come first, in block
// order, and the PULL kernel's warps, which take work in order, then probe
// the rows of about one block at a time, a slice of the DAG small enough to
// stay in L2.  Every other target (few in-edges; its list may need the hash
// table) is grouped over all blocks at once, after all hub groups (see
// PullKeys), so its runs are not split block by block.
constexpr int64_t PL_HUB = (int64_t)PL_WORDS * 32;  // 65536
// tiles per source block: ctx->pull_block_tiles (default 2560 tiles = 10.5M
// edges, 42 MB of adjacency; tc_tuning)
constexpr int PL_MAX_BLOCKS = 64;
// 1: targets outside the hubs are grouped per source block too, so the row
// suffixes their runs probe are a block's rows; 0 (default): over all blocks
// at once, longer runs.  R-MAT scale 24 with 1: 62.96 ms per step against
// 56.22 (pull_kernel 35.2 against 30.4 ms): the extra runs and table builds
// cost more than the L2-resident suffixes save.
#ifndef TC_PL_WIDE_BLOCKS
#define TC_PL_WIDE_BLOCKS 0
#endif
constexpr int64_t PL_LOW_KEY_BUDGET = (int64_t)1 << 28;  // keys of the non-hub part (1 GB of counters)


// pos[key] starts at the exclusive scan of the histogram; each edge takes the
// next slot of its key's group and stores (edge id, row) there
// Record of a grouped edge: (edge id, end of its row) when the DAG is
// relabelled (the probed suffix is (e, rowptr[row + 1])), else (edge id,
// row).  Edges are visited in order, so the row ends are read almost
// sequentially here instead of at random in the probing kernel.
__global__ void __launch_bounds__(PL_GROUP_THREADS) pull_scatter_kernel(const int32_t *__restrict__ col,
                                                                       const int32_t *__restrict__ src,
                                                                       const int64_t *__restrict__ rowptr,
                                                                       int row_end,
                                                                       const int32_t *__restrict__ arm, int64_t m,
                                                                       PullKeys pk,
                                                                       unsigned *__restrict__ pos,
                                                                       uint2 *__restrict__ er) {
  const int64_t T = (m + TILE_EDGES - 1) / TILE_EDGES;
  constexpr int U = PL_SCATTER_UNROLL;  // edges per thread in flight: their atomics overlap
  // tiles in order, or chunks of PL_SCATTER_GRAIN tiles interleaved over the
  // source blocks (see PL_INTERLEAVE)
  const int64_t per = pk.block_edges / TILE_EDGES, S = (T + per - 1) / per;
  const bool il = PL_SCATTER_INTERLEAVE && S > 1 && per % PL_SCATTER_GRAIN == 0;
  const int64_t cpb = per / PL_SCATTER_GRAIN;  // chunks per source block
  for (int64_t i = blockIdx.x; i < (il ? S * per : T); i += gridDim.x) {
    const int64_t c = i / PL_SCATTER_GRAIN;
    const int64_t t = il ? ((c % S) * cpb + c / S) * PL_SCATTER_GRAIN + i % PL_SCATTER_GRAIN : i;
    if (t >= T || arm[t] != TC_ARM_PULL) continue;
    const int64_t e1 = min(m, (t + 1) * TILE_EDGES), kb = pk.block_base(t), lb = pk.low_base(t);
    for (int64_t eb = t * TILE_EDGES + threadIdx.x; eb < e1; eb += U * PL_GROUP_THREADS) {
      int64_t key[U];
      int32_t r[U];
      unsigned slot[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t e = eb + u * PL_GROUP_THREADS;
        key[u] = -1;
        r[u] = 0;
        if (e < e1) {  // read once: streamed past L2, which keeps the counters
          key[u] = pk.key_in(kb, lb, PL_SCATTER_STREAM ? __ldcs(col + e) : __ldg(col + e));
          r[u] = PL_SCATTER_STREAM ? __ldcs(src + e) : __ldg(src + e);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) slot[u] = key[u] >= 0 ? atomicAdd(pos + key[u], 1u) : 0u;
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (key[u] < 0) continue;
        const uint32_t y = row_end ? (uint32_t)__ldg(rowptr + r[u] + 1) : (uint32_t)r[u];
        const uint2 rec = make_uint2((uint32_t)(eb + u * PL_GROUP_THREADS), y);  // one 8-byte store
        if (PL_SCATTER_STREAM) __stcs(er + slot[u], rec);  // evict-first: the counters stay in L2
        else er[slot[u]] = rec;
      }
    }
  }
}

// `er` holds the grouped records (see pull_scatter_kernel); `npull` points
// at their number.
//
// Each warp owns PL_WORDS words of shared memory, all zero between runs, and
// a guard word after them that is never written.  A run of target v uses the
// words as a bitmap over v's id window (min..max of N+(v)) when that window
// has at most PL_WORDS*32 ids, else as a hash table of 4-slot buckets holding
// x+1 (0 = empty; at most two entries per bucket on average) when
// d+(v) <= PL_WORDS/2, else the run's edges fall back to the warp pivot
// search.  Bucket slots fill in order and an entry moves on to the next
// bucket only when all four are taken, so one 16-byte read answers a probe
// unless that bucket is full.  After the run the warp zeroes what it wrote.  A
// bitmap test needs no bounds check: ids outside the window land on zero
// words or, past the table, on the guard word.
constexpr int PL_ROW = PL_WORDS + 4;  // words per warp: table + guard, 16-byte rows

template <bool BITMAP>
__device__ __forceinline__ uint32_t pull_test(const uint32_t *tb, int32_t base, int bits, int32_t x) {
  if (BITMAP) {
    const uint32_t d = (uint32_t)(x - base);
    return (tb[min(d >> 5, (uint32_t)PL_WORDS)] >> (d & 31)) & 1u;
  }
  const uint32_t mask = (1u << bits) - 1u, want = (uint32_t)x + 1u;
  const uint4 *B = reinterpret_cast<const uint4 *>(tb);
  uint32_t b = hslot(x, bits);
  for (;;) {  // ends: the table is at most half full
    const uint4 q = B[b];
    if (q.x == want || q.y == want || q.z == want || q.w == want) return 1u;
    if (q.w == 0u) return 0u;  // bucket never overflowed
    b = (b + 1) & mask;
  }
}

// Grouped entries [k, k2) (one target) against the warp's table: the row
// suffixes of a batch of 32 edges are probed as one flattened sequence of
// 16-byte groups.  Each suffix is widened to the 16-byte blocks that hold it
// (at most 3 entries before and after it; an aligned 16-byte block holding a
// valid entry lies in the same memory page, so the extra reads cannot fault
// and their entries are masked), so no group straddles two edges.  Lane g of
// a pass loads group g (coalesced 16-byte loads, PL_GUNROLL in flight per
// lane) and walks the groups upwards, keeping the edge it is in in registers
// from the batch's prefix sums in shared memory; the next edges' loads issue
// while this one's are tested; the next batch's (edge, row) pairs are
// loaded while this batch probes.  With PER_EDGE each lane sums its hits per
// edge and adds them to the edge's shared counter when it moves on to the
// next edge.
struct PullBatch {
  // per edge of the batch, one 16-byte record read in one load:
  //   x: inclusive prefix sum of the edges' group counts
  //   y: first valid entry of the edge in the batch's entry numbering
  //   z: one past its last valid entry
  //   w: 16-byte block of group g of the edge, counted from the block that
  //      holds col[0]: w + g (fits 32 bits, m < 2^32)
  int4 ed[32];
  uint32_t hits[32];  // PER_EDGE: triangles of each edge of the batch
};

// A grouped record.  TC_PULL_ER_STREAM 1 loads records with evict-first
// hints (they are read in order, about once), leaving L2 to the row
// suffixes and hub bit rows.
#ifndef TC_PULL_ER_STREAM
#define TC_PULL_ER_STREAM 0
#endif
__device__ __forceinline__ uint2 pull_rec(const uint2 *__restrict__ er, int64_t i) {
  return TC_PULL_ER_STREAM ? __ldcs(er + i) : er[i];
}

// Hash runs (targets whose list spans more than the bitmap window) probe
// row suffixes of sources anywhere in the DAG, mostly DRAM misses: with
// TC_PL_HASH_PREFETCH 1 the next batch's suffixes (relabelled DAG: entries
// e + 1 .. row end) are prefetched into L2 while this batch is probed, and
// a pack's before its tables are built, as the 16-byte blocks that hold
// them (the blocks lie in the column array).  Off: at R-MAT scale 24
// pull_kernel took 31.11 ms with it against 30.73 without.
#ifndef TC_PL_HASH_PREFETCH
#define TC_PL_HASH_PREFETCH 0
#endif
__device__ __forceinline__ void prefetch_suffix(const DevDag &g, int64_t e, uint32_t row_end) {
  const int64_t a0 = e + 1;
  if ((int64_t)row_end <= a0) return;
  const uintptr_t lo = reinterpret_cast<uintptr_t>(g.col + a0) & ~(uintptr_t)15;
  const uintptr_t hi = (reinterpret_cast<uintptr_t>(g.col + row_end) + 15) & ~(uintptr_t)15;
  bulk_prefetch_l2(reinterpret_cast<const void *>(lo), (uint32_t)min((uintptr_t)65536, hi - lo));
}

// Dense edges (DENSE, bitmap tables of hub targets only): the table's base is
// hub0 + 128 * woff4, so its 16-byte word j lines up with word woff4 + j of
// every hub bit row; tw4 16-byte words cover it.
struct PullDense {
  int32_t hub0;
  int woff4, tw4;
  int64_t hub_e0;  // first edge of the hub rows (rowptr[hub0])
  int dnum, dden;  // dense when suffix entries * dden > dnum * 32-bit words of the table
};

template <bool BITMAP, bool PER_EDGE, bool TOP, bool DENSE>
__device__ __forceinline__ void pull_run(const DevDag &g, const uint2 *__restrict__ er, int64_t k, int64_t k2,
                                         bool have_b, const uint32_t *tb, int32_t base, int bits, int lane,
                                         PullBatch &sb, uint32_t *out, unsigned long long &acc,
                                         unsigned long long *tile_cycles, unsigned long long build_share,
                                         PullDense pd) {
  int64_t e_n = -1;
  uint32_t y_n = 0;
  if (k + lane < k2) {
    const uint2 p = pull_rec(er, k + lane);
    e_n = p.x;
    y_n = p.y;
  }
  for (int64_t qb = k; qb < k2; qb += 32) {
    const long long t0 = clock64();
    const int64_t e = e_n;
    const uint32_t y = y_n;  // relabelled DAG: end of the edge's row; else its row
    e_n = -1;
    if (qb + 32 + lane < k2) {  // prefetch for the next batch
      const uint2 p = pull_rec(er, qb + 32 + lane);
      e_n = p.x;
      y_n = p.y;
      if (!BITMAP && TC_PL_HASH_PREFETCH && g.restrict_after && have_b) prefetch_suffix(g, e_n, y_n);
    }
    int64_t a0 = 0;
    int na = 0;
    if (e >= 0 && have_b) {
      if (g.restrict_after) {
        a0 = e + 1;
        na = (int)((int64_t)y - a0);
      } else {
        a0 = g.rowptr[y];
        na = (int)(g.rowptr[y + 1] - a0);
      }
    }
    bool dense = false;
    if (DENSE) {  // counted by the word loop below instead of probed; hub rows own edges [hub_e0, m)
      dense = e >= pd.hub_e0 && (int64_t)na * pd.dden > (int64_t)pd.dnum * 4 * pd.tw4;
      if (dense) na = 0;
    }
    const uintptr_t A = reinterpret_cast<uintptr_t>(g.col + a0);
    const int off = na > 0 ? (int)((A >> 2) & 3u) : 0;
    const int ng = na > 0 ? (off + na + 3) >> 2 : 0;
    int gincl = ng;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(TC_FULL_MASK, gincl, o);
      if (lane >= o) gincl += y;
    }
    const int G = __shfl_sync(TC_FULL_MASK, gincl, 31);
    const int gexcl = gincl - ng;
    const uintptr_t col_blk = reinterpret_cast<uintptr_t>(g.col) >> 4;
    sb.ed[lane] = make_int4(gincl, 4 * gexcl + off, 4 * gexcl + off + na, (int)((A >> 4) - col_blk) - gexcl);
    if (PER_EDGE) sb.hits[lane] = 0u;
    __syncwarp();
    int c = 0;
    int4 cur = sb.ed[0];
    uint32_t h = 0;
    int hc = 0;  // PER_EDGE: the edge h belongs to
    for (int gb = 0; gb < G; gb += 32 * PL_GUNROLL) {
      int4 q[PL_GUNROLL];
      int lo[PL_GUNROLL], hi[PL_GUNROLL];  // valid entries of the group: lo <= k < hi
      int ce[PL_GUNROLL];                  // PER_EDGE: edge of the group
      long long gfirst[PL_GUNROLL];        // TOP: DAG entry index of the group's first slot
#pragma unroll
      for (int j = 0; j < PL_GUNROLL; ++j) {
        const int gi = gb + 32 * j + lane;
        q[j] = make_int4(0, 0, 0, 0);
        lo[j] = 0;
        hi[j] = 0;
        if (gi < G) {
          while (gi >= cur.x) cur = sb.ed[++c];  // ends: ed[31].x == G > gi
          q[j] = __ldg(reinterpret_cast<const int4 *>((col_blk + (uintptr_t)(cur.w + gi)) << 4));
          lo[j] = cur.y - 4 * gi;
          hi[j] = cur.z - 4 * gi;
        }
        ce[j] = c;
        if (TOP)
          gfirst[j] = (long long)(((col_blk + (uintptr_t)(cur.w + gi)) << 4) - reinterpret_cast<uintptr_t>(g.col)) >> 2;
      }
#pragma unroll
      for (int j = 0; j < PL_GUNROLL; ++j) {
        if (PER_EDGE && ce[j] != hc) {
          if (h) atomicAdd(&sb.hits[hc], h);
          hc = ce[j];
          h = 0;
        }
        const int32_t xs[4] = {q[j].x, q[j].y, q[j].z, q[j].w};
#pragma unroll
        for (int t = 0; t < 4; ++t)
          if (t >= lo[j] && t < hi[j]) {
            uint32_t hit = pull_test<BITMAP>(tb, base, bits, xs[t]);
            h += hit;
            // the hit closes triangle (u, v, x): entry u->x joins its lowest and highest vertex
            if (TOP && hit) atomicAdd(g.top + gfirst[j] + t, 1u);
          }
      }
    }
    // DENSE: the batch's dense edges, flattened over the lanes as (edge,
    // 16-byte word) pairs, PL_DUNROLL word loads in flight per lane; the
    // per-edge sums go to the edges' hit counters (they have no probe hits)
    uint32_t dc = 0;
    if (DENSE) {
      const unsigned dm = __ballot_sync(TC_FULL_MASK, dense);
      if (dm) {
        if (PER_EDGE && h) {  // flush the probe hits before the records are reused
          atomicAdd(&sb.hits[hc], h);
          h = 0;
        }
        __syncwarp();
        if (dense) sb.ed[__popc(dm & lanemask_lt())] = make_int4(__ldg(g.src + e) - pd.hub0, lane, 0, 0);
        __syncwarp();
        const int nd = __popc(dm), tw4 = pd.tw4;
        const uint4 *t4 = reinterpret_cast<const uint4 *>(tb);
        int d = lane / tw4, j = lane - d * tw4;  // pair lane + 32 i
        int cd = d;
        for (int f0 = 0; f0 < nd * tw4; f0 += 32 * PL_DUNROLL) {
          uint4 a[PL_DUNROLL], b[PL_DUNROLL];
          int du[PL_DUNROLL];
#pragma unroll
          for (int u = 0; u < PL_DUNROLL; ++u) {
            du[u] = d;
            a[u] = make_uint4(0u, 0u, 0u, 0u);
            b[u] = a[u];
            if (d < nd) {
              a[u] = __ldg(g.hub_bits + (size_t)sb.ed[d].x * (size_t)g.hub_wpr4 + pd.woff4 + j);
              b[u] = t4[j];
            }
            j += 32;
            while (j >= tw4) {
              j -= tw4;
              ++d;
            }
          }
#pragma unroll
          for (int u = 0; u < PL_DUNROLL; ++u) {
            const uint32_t x = __popc(a[u].x & b[u].x) + __popc(a[u].y & b[u].y) + __popc(a[u].z & b[u].z) +
                               __popc(a[u].w & b[u].w);
            if (PER_EDGE && du[u] != cd) {
              if (dc) atomicAdd(&sb.hits[sb.ed[cd].y], dc);
              cd = du[u];
              dc = 0;
            }
            dc += x;
          }
        }
        if (PER_EDGE) {
          if (dc && cd < nd) atomicAdd(&sb.hits[sb.ed[cd].y], dc);
          dc = 0;
        }
      }
    }
    if (PER_EDGE) {
      if (h) atomicAdd(&sb.hits[hc], h);
      __syncwarp();
      if (e >= 0) {
        const uint32_t cnt = sb.hits[lane];
        put_edge_count(g, out, e, cnt);
        acc += cnt;
      }
    } else {
      acc += h + dc;
    }
    if (tile_cycles) {  // share of this batch's time by the edge's probe count, plus the build share
      const unsigned tot = __reduce_add_sync(TC_FULL_MASK, (unsigned)(e >= 0 ? na + 1 : 0));
      if (e >= 0) {
        const unsigned long long dt = (unsigned long long)(clock64() - t0);
        atomicAdd(&tile_cycles[e / TILE_EDGES], dt * (unsigned long long)(na + 1) / tot + build_share);
      }
    }
    __syncwarp();
  }
}

// Packed hash runs.  Most targets whose list needs the hash table have few
// in-edges (at R-MAT scale 22 half of them have at most 3), and each run pays
// a chain of dependent loads (record, target, row pointers, list ends, list)
// before its one or two probe passes.  When a run of a hash target ends
// inside the first 32 records, the following complete runs of hash targets
// in those 32 records (lists of at most PK_NB entries) are counted with it:
// each gets its own hash table, carved from the warp's words (at most
// PK_TSEL words in all), the lists are inserted as one flattened sequence,
// and the <= 32 edges are probed as one batch, each edge testing its own
// run's table.  The words [PK_TSEL, PL_WORDS) hold each edge's table
// (word offset | bits << 16) during the batch.
#ifndef TC_PL_PACK
#define TC_PL_PACK 1
#endif
constexpr int PK_NB = 256;
#ifndef TC_PK_LOAD
#define TC_PK_LOAD 1  // 1 or 2: a table then is at most a quarter or half full
#endif
constexpr int PK_LOAD = TC_PK_LOAD;  // packed tables: entries per bucket on average (1 or 2)
static_assert(PK_LOAD == 1 || PK_LOAD == 2, "a packed table must keep a free slot");
constexpr int PK_TSEL = PL_WORDS - 32;

// Lane j stands for record k + j; `v` is record k's target and `vw` the
// target of record k + 1 + lane (-1 past p1).  Returns the end of the packed
// records, or k when fewer than two runs qualify (nothing was done).
template <bool PER_EDGE>
__device__ __forceinline__ int64_t pull_pack(const DevDag &g, const uint2 *__restrict__ er, int64_t k, int64_t p1,
                                             int32_t v, int32_t vw, uint32_t *tb, int lane, PullBatch &sb,
                                             uint32_t *out, unsigned long long &acc,
                                             unsigned long long *tile_cycles) {
  const long long t0 = clock64();
  const bool valid = k + lane < p1;
  int32_t tgt = __shfl_up_sync(TC_FULL_MASK, vw, 1);
  if (lane == 0) tgt = v;
  const int32_t prev = __shfl_up_sync(TC_FULL_MASK, tgt, 1);
  const bool start = valid && (lane == 0 || tgt != prev);
  const unsigned E = __ballot_sync(TC_FULL_MASK, valid && vw != tgt);  // last record of its run
  int nb = 0, words = 0, bits = 3;
  int64_t bb = 0;
  bool ok = false;
  if (start && (E >> lane) != 0u) {  // the run ends inside the window
    bb = g.rowptr[tgt];
    nb = (int)(g.rowptr[tgt + 1] - bb);
    if (nb > 0 && nb <= PK_NB) {
      const uint32_t span = (uint32_t)(__ldg(g.col + bb + nb - 1) - __ldg(g.col + bb)) + 1u;
      if (span > (uint32_t)PL_WORDS * 32u) {  // a hash target, as in the single-run rule
        while ((1 << bits) < (nb + PK_LOAD - 1) / PK_LOAD) ++bits;  // at most PK_LOAD entries per 4-slot bucket on average
        words = 4 << bits;
        ok = true;
      }
    }
  }
  const unsigned bad = __ballot_sync(TC_FULL_MASK, start && !ok);
  const unsigned below = bad ? (1u << (__ffs(bad) - 1)) - 1u : 0xffffffffu;  // lanes before the first misfit
  int wi = ok ? words : 0, ni = ok ? nb : 0;  // inclusive sums over the runs
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int a = __shfl_up_sync(TC_FULL_MASK, wi, o), b = __shfl_up_sync(TC_FULL_MASK, ni, o);
    if (lane >= o) {
      wi += a;
      ni += b;
    }
  }
  const unsigned inc = __ballot_sync(TC_FULL_MASK, start) & below & __ballot_sync(TC_FULL_MASK, wi <= PK_TSEL);
  if (__popc(inc) < 2) return k;
  const int L = 31 - __clz(inc);                       // start of the last packed run
  const int ne = __ffs(E & ~((1u << L) - 1u));         // records in the pack: through that run's end
  const int tot_words = __shfl_sync(TC_FULL_MASK, wi, L), tot_nb = __shfl_sync(TC_FULL_MASK, ni, L);
  // per run: (inclusive entry sum, table word offset | bits << 16, list base
  // such that pack entry i is col[base + i])
  if ((inc >> lane) & 1u) {
    const int64_t base = bb - (int64_t)(ni - nb);
    sb.ed[__popc(inc & lanemask_lt())] =
        make_int4(ni, (wi - words) | (bits << 16), (int)(uint32_t)(uint64_t)base, (int)((uint64_t)base >> 32));
  }
  // the pack's records first, so that (hash-run prefetch) their row
  // suffixes are on the way to L2 while the tables are built
  const bool mine = lane < ne;
  int64_t e = -1;
  uint32_t y = 0;
  if (mine) {
    const uint2 p = pull_rec(er, k + lane);
    e = p.x;
    y = p.y;
    if (TC_PL_HASH_PREFETCH && g.restrict_after) prefetch_suffix(g, e, y);
  }
  __syncwarp();
  {  // build: the runs' lists as one flattened sequence, PL_UNROLL loads in flight per lane
    int c = 0;
    int4 cur = sb.ed[0];
    for (int q0 = 0; q0 < tot_nb; q0 += 32 * PL_UNROLL) {
      int32_t x[PL_UNROLL];
      uint32_t ts[PL_UNROLL];
#pragma unroll
      for (int u = 0; u < PL_UNROLL; ++u) {
        const int i = q0 + 32 * u + lane;
        x[u] = 0;
        ts[u] = 0u;
        if (i < tot_nb) {
          while (i >= cur.x) cur = sb.ed[++c];  // ends: the last run's sum is tot_nb > i
          const int64_t base = (int64_t)(((uint64_t)(uint32_t)cur.w << 32) | (uint64_t)(uint32_t)cur.z);
          x[u] = __ldg(g.col + base + i);
          ts[u] = (uint32_t)cur.y;
        }
      }
#pragma unroll
      for (int u = 0; u < PL_UNROLL; ++u) {
        if (q0 + 32 * u + lane >= tot_nb) continue;
        uint32_t *T = tb + (ts[u] & 0xffffu);
        const int tbits = (int)(ts[u] >> 16);
        const uint32_t mask = (1u << tbits) - 1u, val = (uint32_t)x[u] + 1u;
        uint32_t b = hslot(x[u], tbits);
        for (;;) {  // ends: every table is at most half full (PK_LOAD <= 2)
          uint32_t *bk = T + 4 * b;
          if (atomicCAS(bk, 0u, val) == 0u || atomicCAS(bk + 1, 0u, val) == 0u || atomicCAS(bk + 2, 0u, val) == 0u ||
              atomicCAS(bk + 3, 0u, val) == 0u)
            break;
          b = (b + 1) & mask;
        }
      }
    }
  }
  __syncwarp();
  const uint32_t tsel = mine ? (uint32_t)sb.ed[__popc(inc & (lanemask_lt() | (1u << lane))) - 1].y : 0u;
  int64_t a0 = 0;
  int na = 0;
  if (mine) {
    if (g.restrict_after) {
      a0 = e + 1;
      na = (int)((int64_t)y - a0);
    } else {
      a0 = g.rowptr[y];
      na = (int)(g.rowptr[y + 1] - a0);
    }
  }
  // the batch's records, as in pull_run
  const uintptr_t A = reinterpret_cast<uintptr_t>(g.col + a0);
  const int off = na > 0 ? (int)((A >> 2) & 3u) : 0;
  const int ng = na > 0 ? (off + na + 3) >> 2 : 0;
  int gincl = ng;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(TC_FULL_MASK, gincl, o);
    if (lane >= o) gincl += t;
  }
  const int G = __shfl_sync(TC_FULL_MASK, gincl, 31);
  const int gexcl = gincl - ng;
  const uintptr_t col_blk = reinterpret_cast<uintptr_t>(g.col) >> 4;
  __syncwarp();  // every lane has read its run's table from sb.ed
  sb.ed[lane] = make_int4(gincl, 4 * gexcl + off, 4 * gexcl + off + na, (int)((A >> 4) - col_blk) - gexcl);
  tb[PK_TSEL + lane] = tsel;
  if (PER_EDGE) sb.hits[lane] = 0u;
  __syncwarp();
  int c = 0;
  int4 cur = sb.ed[0];
  uint32_t cts = tb[PK_TSEL];
  uint32_t h = 0;
  int hc = 0;
  for (int gb = 0; gb < G; gb += 32 * PL_GUNROLL) {
    int4 q[PL_GUNROLL];
    int lo[PL_GUNROLL], hi[PL_GUNROLL], ce[PL_GUNROLL];
    uint32_t ts[PL_GUNROLL];
#pragma unroll
    for (int j = 0; j < PL_GUNROLL; ++j) {
      const int gi = gb + 32 * j + lane;
      q[j] = make_int4(0, 0, 0, 0);
      lo[j] = 0;
      hi[j] = 0;
      if (gi < G) {
        while (gi >= cur.x) {  // ends: ed[31].x == G > gi
          cur = sb.ed[++c];
          cts = tb[PK_TSEL + c];
        }
        q[j] = __ldg(reinterpret_cast<const int4 *>((col_blk + (uintptr_t)(cur.w + gi)) << 4));
        lo[j] = cur.y - 4 * gi;
        hi[j] = cur.z - 4 * gi;
      }
      ce[j] = c;
      ts[j] = cts;
    }
#pragma unroll
    for (int j = 0; j < PL_GUNROLL; ++j) {
      if (PER_EDGE && ce[j] != hc) {
        if (h) atomicAdd(&sb.hits[hc], h);
        hc = ce[j];
        h = 0;
      }
      const int32_t xs[4] = {q[j].x, q[j].y, q[j].z, q[j].w};
#pragma unroll
      for (int t = 0; t < 4; ++t)
        if (t >= lo[j] && t < hi[j]) h += pull_test<false>(tb + (ts[j] & 0xffffu), 0, (int)(ts[j] >> 16), xs[t]);
    }
  }
  if (PER_EDGE) {
    if (h) atomicAdd(&sb.hits[hc], h);
    __syncwarp();
    if (mine) {
      const uint32_t cnt = sb.hits[lane];
      put_edge_count(g, out, e, cnt);
      acc += cnt;
    }
  } else {
    acc += h;
  }
  if (tile_cycles) {  // the pack's time, shared by the edges' probe counts
    const unsigned tot = __reduce_add_sync(TC_FULL_MASK, (unsigned)(mine ? na + 1 : 0));
    if (mine) {
      const unsigned long long dt = (unsigned long long)(clock64() - t0);
      atomicAdd(&tile_cycles[e / TILE_EDGES], dt * (unsigned long long)(na + 1) / tot);
    }
  }
  __syncwarp();
  // back to all zero: the tables and the per-edge table words
  uint4 *t4 = reinterpret_cast<uint4 *>(tb);
  for (int q2 = lane; q2 < (tot_words >> 2); q2 += 32) t4[q2] = make_uint4(0u, 0u, 0u, 0u);
  if (lane < 8) t4[(PK_TSEL >> 2) + lane] = make_uint4(0u, 0u, 0u, 0u);
  __syncwarp();
  return k + ne;
}

// Work is taken in chunks of grouped entries that shrink from `item` to
// `item_min` as the remaining work falls, so the last chunks end together
// (the ctx's pull_item / pull_item_min; 512 and 128 unless tuned).
__device__ __forceinline__ unsigned pull_next_chunk(unsigned *head, int64_t np, int64_t warps, int item,
                                                    int item_min, int64_t *end) {
  const int64_t seen = (int64_t)*(volatile unsigned *)head;
  const int64_t left = np - seen;
  int64_t chunk = left / warps;
  chunk = chunk >= item ? item : chunk <= item_min ? item_min : chunk;
  const unsigned start = atomicAdd(head, (unsigned)chunk);
  *end = min(np, (int64_t)start + chunk);
  return start;
}

// MODE 1: per-vertex counts (g.top set, per-edge output); MODE 2: labelled
// counts (g.vlabel set).  Separate instantiations, so the plain kernel
// (MODE 0) keeps its registers.
template <int MODE>
__global__ void __launch_bounds__(PL_THREADS, TC_PL_MIN_BLOCKS) pull_kernel(DevDag g, const uint2 *__restrict__ er,
                                                         const unsigned *__restrict__ npull,
                                                         unsigned *head, uint32_t *out, unsigned long long *total,
                                                         unsigned long long *tile_cycles, int item, int item_min,
                                                         int dense_num, int dense_den) {
  __shared__ __align__(16) uint32_t tab[PL_WARPS][PL_ROW];
  __shared__ PullBatch s_batch[PL_WARPS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t *tb = tab[w];
  for (int q = lane; q < PL_ROW; q += 32) tb[q] = 0u;
  __syncwarp();
  const int64_t np = (int64_t)*npull;
  const int64_t warps = (int64_t)gridDim.x * PL_WARPS;
  const int32_t hub0 = (int32_t)(g.n - (g.n < PL_DENSE_HUB ? g.n : PL_DENSE_HUB));  // dense edges' hubs
  const int64_t hub_e0 = g.hub_bits != nullptr ? g.rowptr[hub0] : g.m;
  unsigned long long acc = 0;
  for (;;) {
    unsigned it = 0;
    int64_t p1 = 0;
    if (lane == 0) it = pull_next_chunk(head, np, warps, item, item_min, &p1);
    it = __shfl_sync(TC_FULL_MASK, it, 0);
    p1 = __shfl_sync(TC_FULL_MASK, (long long)p1, 0);
    if ((int64_t)it >= np) break;
    const int64_t p0 = (int64_t)it;
    for (int64_t k = p0; k < p1;) {
      const long long tr0 = clock64();  // profiling: the run's search and table build are its edges' cost too
      const int32_t v = __ldg(g.col + pull_rec(er, k).x);
      // end of the run of target v inside this chunk; vw keeps the targets of
      // records k + 1 .. k + 32 for packing short hash runs
      int64_t k2 = k + 1;
      int32_t vw = -1;
      for (bool first = true;; first = false) {
        const int64_t j = k2 + lane;
        const int32_t vj = j < p1 ? __ldg(g.col + pull_rec(er, j).x) : -1;
        if (first) vw = vj;
        const unsigned bal = __ballot_sync(TC_FULL_MASK, vj != v);
        if (bal) { k2 += __ffs(bal) - 1; break; }
        k2 += 32;
      }
      const int64_t bb = g.rowptr[v];
      const int nb = (int)(g.rowptr[v + 1] - bb);
      int32_t bmin = nb > 0 ? __ldg(g.col + bb) : 0;
      uint32_t span = nb > 0 ? (uint32_t)(__ldg(g.col + bb + nb - 1) - bmin) + 1u : 0u;
      const bool bitmap = span <= (uint32_t)PL_WORDS * 32u;
#if TC_PL_PACK
      if (MODE == 0 && !bitmap && nb <= PK_NB && k2 <= k + 32 && k2 < p1) {  // a short hash run: pack it
        const int64_t kp = out == nullptr ? pull_pack<false>(g, er, k, p1, v, vw, tb, lane, s_batch[w], out, acc,
                                                             tile_cycles)
                                          : pull_pack<true>(g, er, k, p1, v, vw, tb, lane, s_batch[w], out, acc,
                                                            tile_cycles);
        if (kp > k) {
          k = kp;
          continue;
        }
      }
#endif
      // dense edges need the table aligned with the hub bit rows: the base goes
      // down to a 128-id boundary counted from hub0 (a hub target's list lies
      // in (v, n), so the window still fits)
      PullDense pd{hub0, 0, 0, hub_e0, dense_num, dense_den};
      bool dense_run = MODE != 1 && g.hub_bits != nullptr && bitmap && nb > 0 && v >= hub0;
      if (dense_run) {
        const int32_t bmax = bmin + (int32_t)span - 1;
        const int woff4 = (bmin - hub0) >> 7;
        const uint32_t span2 = (uint32_t)(bmax - (hub0 + 128 * woff4)) + 1u;
        if (span2 <= (uint32_t)PL_WORDS * 32u) {  // the aligned window still fits the table
          pd.woff4 = woff4;
          bmin = hub0 + 128 * woff4;
          span = span2;
          pd.tw4 = (int)((span + 127u) >> 7);
        } else {
          dense_run = false;
        }
      }
      if (!bitmap && nb > PL_WORDS / 2) {  // wide window and long list: warp pivot search per edge
        long long tq = tr0;
        for (int64_t q = k; q < k2; ++q) {
          const int64_t e = pull_rec(er, q).x;
          int32_t s;
          const EdgeLists L = edge_lists(g, e, s);
          uint32_t c = 0;
          if (L.na > 0 && L.nb > 0) {
            if (MODE != 0)
              c = attr_search_count(L.a, L.na, L.b, L.nb, MODE == 1 ? g.top + (L.a - g.col) : nullptr,
                                    MODE == 2 ? g.vlabel : nullptr, g.label, lane);
            else if (L.na <= L.nb) c = pivot_search_count(L.a, L.na, L.b, L.nb, lane);
            else c = pivot_search_count(L.b, L.nb, L.a, L.na, lane);
          }
          c = warp_sum(c);
          if (lane == 0) {
            put_edge_count(g, out, e, c);
            acc += c;
            if (tile_cycles) {
              const long long now = clock64();
              atomicAdd(&tile_cycles[e / TILE_EDGES], (unsigned long long)(now - tq));
              tq = now;
            }
          }
        }
        k = k2;
        continue;
      }
      int bits = 3;  // hash mode: log2 of the bucket count, one bucket per entry up to 512 entries
      if (!bitmap)
        while ((1 << bits) < nb && (8 << bits) <= PL_WORDS) ++bits;
      // build: PL_UNROLL list loads in flight per lane
      for (int q0 = 0; q0 < nb; q0 += 32 * PL_UNROLL) {
        int32_t x[PL_UNROLL];
#pragma unroll
        for (int u = 0; u < PL_UNROLL; ++u) {
          const int q = q0 + 32 * u + lane;
          x[u] = q < nb ? __ldg(g.col + bb + q) : 0;
        }
#pragma unroll
        for (int u = 0; u < PL_UNROLL; ++u) {
          if (q0 + 32 * u + lane >= nb) continue;
          // labelled counts: the table holds only N+(v)'s entries with the
          // label, so every hit is a labelled one (no test per probe)
          if (MODE == 2 && g.vlabel[x[u]] != g.label) continue;
          if (bitmap) {
            const uint32_t d = (uint32_t)(x[u] - bmin);
            if (d < span) atomicOr(&tb[d >> 5], 1u << (d & 31));  // false only for an unsorted list
          } else {  // first free slot of the first bucket with room
            const uint32_t mask = (1u << bits) - 1u;
            uint32_t b = hslot(x[u], bits);
            for (;;) {
              uint32_t *bk = tb + 4 * b;
              if (atomicCAS(bk, 0u, (uint32_t)x[u] + 1u) == 0u || atomicCAS(bk + 1, 0u, (uint32_t)x[u] + 1u) == 0u ||
                  atomicCAS(bk + 2, 0u, (uint32_t)x[u] + 1u) == 0u || atomicCAS(bk + 3, 0u, (uint32_t)x[u] + 1u) == 0u)
                break;
              b = (b + 1) & mask;
            }
          }
        }
      }
      __syncwarp();
      const unsigned long long build_share =
          tile_cycles ? (unsigned long long)(clock64() - tr0) / (unsigned long long)(k2 - k) : 0ull;
      if (MODE == 1) {  // per-vertex counts: per-edge output plus the top-edge attribution
        if (bitmap)
          pull_run<true, true, true, false>(g, er, k, k2, nb > 0, tb, bmin, bits, lane, s_batch[w], out, acc,
                                                   tile_cycles, build_share, pd);
        else
          pull_run<false, true, true, false>(g, er, k, k2, nb > 0, tb, bmin, bits, lane, s_batch[w], out, acc,
                                                    tile_cycles, build_share, pd);
      } else if (out == nullptr) {  // total only
        if (dense_run)
          pull_run<true, false, false, MODE != 1>(g, er, k, k2, true, tb, bmin, bits, lane, s_batch[w], out,
                                                         acc, tile_cycles, build_share, pd);
        else if (bitmap)
          pull_run<true, false, false, false>(g, er, k, k2, nb > 0, tb, bmin, bits, lane, s_batch[w], out, acc,
                                                   tile_cycles, build_share, pd);
        else
          pull_run<false, false, false, false>(g, er, k, k2, nb > 0, tb, bmin, bits, lane, s_batch[w], out, acc,
                                                    tile_cycles, build_share, pd);
      } else if (dense_run) {
        pull_run<true, true, false, MODE != 1>(g, er, k, k2, true, tb, bmin, bits, lane, s_batch[w], out, acc,
                                                      tile_cycles, build_share, pd);
      } else if (bitmap) {
        pull_run<true, true, false, false>(g, er, k, k2, nb > 0, tb, bmin, bits, lane, s_batch[w], out, acc,
                                                tile_cycles, build_share, pd);
      } else {
        pull_run<false, true, false, false>(g, er, k, k2, nb > 0, tb, bmin, bits, lane, s_batch[w], out, acc,
                                                 tile_cycles, build_share, pd);
      }
      __syncwarp();
      // back to all zero: the touched word range with 16-byte stores, or the
      // list's own words when the window is much wider than the list
      const int words = bitmap ? (int)((span + 31u) >> 5) : (4 << bits);
      if (!bitmap || words <= 16 * nb) {
        uint4 *t4 = reinterpret_cast<uint4 *>(tb);
        for (int q = lane; q < (words + 3) >> 2; q += 32) t4[q] = make_uint4(0u, 0u, 0u, 0u);
      } else {
        for (int q = lane; q < nb; q += 32) {
          const uint32_t d = (uint32_t)(__ldg(g.col + bb + q) - bmin);
          if (d < span) tb[d >> 5] = 0u;
        }
      }
      __syncwarp();
      k = k2;
    }
  }
  flush_total(acc, total);
}

// ---- host side ---------------------------------------------------------------------

typedef void (*ArmKernel)(DevDag, const uint32_t *, const int64_t *, int, unsigned *, uint32_t *,
                          unsigned long long *, unsigned long long *);

static ArmKernel arm_kernel(int arm) {
  switch (arm) {
    case TC_ARM_BSEARCH_4: return bsearch_kernel<4>;
#if TC_BS32_PIVOT
    case TC_ARM_BSEARCH_32: return bsearch_kernel<32>;
#else
    case TC_ARM_BSEARCH_32: return bsearch_tma_kernel;
#endif
    case TC_ARM_MERGE_8: return merge_kernel<8>;
    case TC_ARM_MERGE_32: return merge_kernel<32>;
    case TC_ARM_HASH: return hash_kernel;
    case TC_ARM_GALLOP_4: return gallop_kernel<4>;
    case TC_ARM_MPATH_2: return mpath_kernel<2>;
    case TC_ARM_FLAT: return flat_kernel;
    default: return bitmap_kernel;
  }
}
static const void *arm_func(int arm) {
  return arm == TC_ARM_PULL ? (const void *)pull_kernel<0> : (const void *)arm_kernel(arm);
}
static int arm_threads(int arm) {
  return arm == TC_ARM_BITMAP ? BM_THREADS : arm == TC_ARM_HASH ? HT_THREADS : arm == TC_ARM_PULL ? PL_THREADS : CT_THREADS;
}
static int arm_smem(int arm) { return arm == TC_ARM_BITMAP ? BM_SMEM_BYTES : 0; }

tc_status init_arm_occupancy(tc_ctx *ctx) {
  TC_CHECK_CUDA(ctx, cudaFuncSetAttribute(bitmap_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, BM_SMEM_BYTES));
  TC_CHECK_CUDA(ctx, cudaFuncSetAttribute(plan_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)(TC_MLP_PARAM_COUNT * sizeof(float))));
  for (int a = 0; a < TC_NUM_ARMS; ++a) {
    int nb = 0;
    TC_CHECK_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, arm_func(a), arm_threads(a), arm_smem(a)));
    ctx->arm_blocks_per_sm[a] = nb > 0 ? nb : 1;
    // independent workers per SM: warps for the warp-level arms, blocks otherwise
    const bool warp_items = a == TC_ARM_HASH || a == TC_ARM_FLAT || a == TC_ARM_PULL;
    ctx->arm_units_per_sm[a] = ctx->arm_blocks_per_sm[a] * (warp_items ? arm_threads(a) / 32 : 1);
  }
  return TC_OK;
}

static int64_t pull_key_count(int64_t n, int64_t T, int block_tiles, PullKeys *pk);

static size_t count_sort_scratch_bytes(const tc_ctx *ctx, int64_t n, int64_t T) {
  return std::max(radix_sort_scratch_bytes(ctx, T > 0 ? T : 1), scan_scratch_bytes(ctx, pull_key_count(n, T, ctx->pull_block_tiles, nullptr) + 1));
}

// Hub bit rows: one row per dense hub (the top min(n, PL_DENSE_HUB) ids), each
// hub_wpr4(n) 16-byte words wide (one bit per hub id).
static int64_t hub_rows(int64_t n) { return std::min<int64_t>(n, PL_DENSE_HUB); }
static int hub_wpr4(int64_t n) { return (int)((hub_rows(n) + 127) / 128); }
static int64_t hub_bits_words4(int64_t n) { return hub_rows(n) * hub_wpr4(n); }

size_t count_scratch_bytes(const tc_ctx *ctx, int64_t n, int64_t m) {
  const int64_t T = (m + TILE_EDGES - 1) / TILE_EDGES;
  Sizer sz;
  sz.take<float>(T * TC_MLP_FEATURES);
  sz.take<uint64_t>(T);
  sz.take<uint64_t>(T);
  sz.take<uint32_t>(T);
  sz.take<uint32_t>(T);
  sz.take<int32_t>(T);
  sz.take<int64_t>(TC_NUM_ARMS + 1);
  sz.take<unsigned long long>(T);
  sz.take<unsigned long long>(T);
  sz.take<unsigned long long>(TC_NUM_ARMS);
  sz.take<uint32_t>(pull_key_count(n, T, ctx->pull_block_tiles, nullptr) + 1);
  sz.take<uint2>(m);
  sz.take<uint4>(hub_bits_words4(n));
  return sz.used + count_sort_scratch_bytes(ctx, n, T) + 256;
}

tc_status count_carve(const tc_ctx *ctx, int64_t n, int64_t m, Bump &bump, CountBufs &cb, bool want_cycles) {
  const int64_t T = (m + TILE_EDGES - 1) / TILE_EDGES;
  cb.features = bump.take<float>(T * TC_MLP_FEATURES);
  cb.qkeys0 = bump.take<uint64_t>(T);
  cb.qkeys1 = bump.take<uint64_t>(T);
  cb.qvals0 = bump.take<uint32_t>(T);
  cb.qvals1 = bump.take<uint32_t>(T);
  cb.arm = bump.take<int32_t>(T);
  cb.qoff = bump.take<int64_t>(TC_NUM_ARMS + 1);
  unsigned long long *cyc = bump.take<unsigned long long>(T);
  cb.tile_cycles = want_cycles ? cyc : nullptr;
  cb.tile_bytes = bump.take<unsigned long long>(T);
  cb.arm_bytes = bump.take<unsigned long long>(TC_NUM_ARMS);
  cb.pull_pos = bump.take<uint32_t>(pull_key_count(n, T, ctx->pull_block_tiles, nullptr) + 1);
  cb.pull_er = bump.take<uint2>(m);
  cb.hub_bits = bump.take<uint4>(hub_bits_words4(n));
  cb.sort_scratch = bump.take<char>((int64_t)count_sort_scratch_bytes(ctx, n, T));
  return bump.overflow ? TC_ERR_OOM : TC_OK;
}

// Pinned host scratch layout used by run_count / count_stats (64 words).
constexpr int PIN_QOFF = 16;                           // TC_NUM_ARMS + 1 int64
constexpr int PIN_BYTES = PIN_QOFF + TC_NUM_ARMS + 1;  // TC_NUM_ARMS uint64
constexpr int PIN_PULL = PIN_BYTES + TC_NUM_ARMS;       // uint32: edges the PULL arm grouped
static_assert(PIN_BYTES + TC_NUM_ARMS <= 64, "pinned scratch holds 64 words");
static_assert(sizeof(((tc_ctx *)nullptr)->ev) / sizeof(cudaEvent_t) >= 10 + TC_NUM_ARMS, "one event per arm");

// Number of keys of the PULL grouping of a graph with n vertices and T tiles.
// The non-hub part takes hub0 keys per block; its blocks are the hub part's
// (TC_PL_WIDE_BLOCKS 1) as far as PL_LOW_KEY_BUDGET keys allow, else coarser.
static int64_t pull_key_count(int64_t n, int64_t T, int block_tiles, PullKeys *pk) {
  const int64_t per_block = std::max<int64_t>(block_tiles, (T + PL_MAX_BLOCKS - 1) / PL_MAX_BLOCKS);
  const int64_t blocks = std::max<int64_t>(1, (T + per_block - 1) / per_block);
  const int64_t hub0 = n - std::min<int64_t>(n, PL_HUB);
  int64_t low_blocks = 1;
  if (TC_PL_WIDE_BLOCKS && hub0 > 0)
    low_blocks = std::max<int64_t>(1, std::min<int64_t>(blocks, PL_LOW_KEY_BUDGET / hub0));
  const int64_t low_per_block = std::max<int64_t>(1, (T + low_blocks - 1) / low_blocks);
  low_blocks = std::max<int64_t>(1, (T + low_per_block - 1) / low_per_block);
  if (pk) {
    pk->hub_span = PL_HUB;
    pk->hub0 = hub0;
    pk->block_edges = per_block * TILE_EDGES;
    pk->global0 = blocks * PL_HUB;
    pk->low_block_edges = low_per_block * TILE_EDGES;
  }
  return blocks * PL_HUB + low_blocks * hub0;
}

// PULL arm: group the PULL tiles' edges (one counting sort: plan_kernel
// counted the keys), then count.  The scatter kernel runs over every tile
// (each block skips tiles of other arms) since the number of PULL tiles is
// known only on the device.
#ifndef TC_HUB_BITS_SCAN
#define TC_HUB_BITS_SCAN 1
#endif
// Bit rows of the hubs' out-lists, one warp per hub row: the warp clears the
// row, then ORs in its entries, one OR per distinct word (lanes matched by
// word).  Every entry of a hub row is a hub (it ranks above its row).  Nothing
// is done when no edge was grouped for the PULL arm.
__global__ void hub_bits_kernel(DevDag g, int32_t hub0, int wpr4, const unsigned *__restrict__ npull,
                                uint4 *__restrict__ bits) {
  if (*npull == 0) return;
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < g.n - hub0; row += warps) {
    uint4 *b4 = bits + row * wpr4;
    for (int q = lane; q < wpr4; q += 32) b4[q] = make_uint4(0u, 0u, 0u, 0u);
    __syncwarp();
    uint32_t *b = reinterpret_cast<uint32_t *>(b4);
    const int64_t e0 = g.rowptr[hub0 + row], e1 = g.rowptr[hub0 + row + 1];
    for (int64_t e = e0 + lane; e - lane < e1; e += 32) {
      const bool in = e < e1;
      const int32_t w = in ? g.col[e] - hub0 : -1;
      const bool ok = in && w >= 0;  // false only outside a relabelled DAG
#if TC_HUB_BITS_SCAN
      // the row is sorted, so lanes sharing a word are a run: a segmented OR
      // scan leaves the run's bits in its last lane, which stores them
      // (for any order every bit still reaches the last lane of its run)
      const int wid = ok ? (w >> 5) : -1;
      unsigned x = ok ? 1u << (w & 31) : 0u;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(TC_FULL_MASK, x, o);
        const int wy = __shfl_up_sync(TC_FULL_MASK, wid, o);
        if (lane >= o && wy == wid) x |= y;
      }
      const int wn = __shfl_down_sync(TC_FULL_MASK, wid, 1);
      if (ok && (lane == 31 || wn != wid)) atomicOr(b + wid, x);
#else
      const unsigned act = __ballot_sync(TC_FULL_MASK, ok);
      if (ok) {
        const unsigned peers = __match_any_sync(act, w >> 5);
        const unsigned word = __reduce_or_sync(peers, 1u << (w & 31));
        if (lane == __ffs(peers) - 1) atomicOr(b + (w >> 5), word);
      }
#endif
    }
    __syncwarp();
  }
}

static tc_status run_pull(tc_ctx *ctx, const DevDag &g_in, CountBufs &cb, uint32_t *out, int64_t T, bool timing) {
  PullKeys pk;
  const int64_t K = pull_key_count(g_in.n, T, ctx->pull_block_tiles, &pk);
  unsigned *pos = cb.pull_pos;
  const int gblocks = (int)std::min<int64_t>(T, (int64_t)ctx->num_sms * 8);
  TC_TRY(exclusive_scan_u32(ctx, cb.pull_pos, cb.pull_pos, K + 1, cb.sort_scratch));
  pull_scatter_kernel<<<gblocks, PL_GROUP_THREADS, 0, ctx->stream>>>(g_in.col, g_in.src, g_in.rowptr,
                                                                     g_in.restrict_after, cb.arm, g_in.m, pk, pos,
                                                                     cb.pull_er);
  TC_CHECK_LAUNCH(ctx);
  DevDag g = g_in;
  // dense edges: plain and labelled counts of a relabelled DAG (rows hold
  // higher ids only; labelled tables hold only the labelled entries)
  if (g.restrict_after && !g.top && g.m > 0) {
    const int32_t hub0 = (int32_t)(g.n - hub_rows(g.n));
    hub_bits_kernel<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(g, hub0, hub_wpr4(g.n), pos + K, cb.hub_bits);
    TC_CHECK_LAUNCH(ctx);
    g.hub_bits = cb.hub_bits;
    g.hub_wpr4 = hub_wpr4(g.n);
  }
  // pos[K] (no edge has key K) still holds the number of grouped edges
  const int grid = ctx->num_sms * ctx->arm_blocks_per_sm[TC_ARM_PULL];
  if (timing) {
    TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ctx->h_pinned[PIN_PULL], pos + K, sizeof(unsigned), cudaMemcpyDeviceToHost,
                                       ctx->stream));
    TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[10 + TC_NUM_ARMS], ctx->stream));
  }
  if (g.top)
    pull_kernel<1><<<grid, PL_THREADS, 0, ctx->stream>>>(g, cb.pull_er, pos + K, ctx->d_heads + TC_ARM_PULL, out,
                                                        ctx->d_total, cb.tile_cycles, ctx->pull_item,
                                                        ctx->pull_item_min, ctx->pull_dense_num, ctx->pull_dense_den);
  else if (g.vlabel)
    pull_kernel<2><<<grid, PL_THREADS, 0, ctx->stream>>>(g, cb.pull_er, pos + K, ctx->d_heads + TC_ARM_PULL, out,
                                                        ctx->d_total, cb.tile_cycles, ctx->pull_item,
                                                        ctx->pull_item_min, ctx->pull_dense_num, ctx->pull_dense_den);
  else
    pull_kernel<0><<<grid, PL_THREADS, 0, ctx->stream>>>(g, cb.pull_er, pos + K,
                                                    ctx->d_heads + TC_ARM_PULL, out, ctx->d_total, cb.tile_cycles, ctx->pull_item,
                                                        ctx->pull_item_min, ctx->pull_dense_num, ctx->pull_dense_den);
  TC_CHECK_LAUNCH(ctx);
  if (timing) {
    TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[11 + TC_NUM_ARMS], ctx->stream));
    ctx->pull_timed = true;
  }
  return TC_OK;
}

tc_status run_count(tc_ctx *ctx, const DevDag &g_in, const tc_opts &opts, CountBufs &cb, uint32_t *out, bool timing) {
  DevDag g = g_in;
  g.flags = ctx->d_flags;
  const int64_t T = (g.m + TILE_EDGES - 1) / TILE_EDGES;
  if (opts.selector == TC_SELECT_LEARNED && !ctx->mlp_loaded)
    return set_error(ctx, TC_ERR_INVALID_ARG, "learned selector requested but no MLP weights are loaded");
  if (opts.selector == TC_SELECT_FORCE && (opts.force_arm < 0 || opts.force_arm >= TC_NUM_ARMS))
    return set_error(ctx, TC_ERR_INVALID_ARG, "force_arm %d outside [0,%d)", opts.force_arm, TC_NUM_ARMS);
  if (timing) TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[8], ctx->stream));
  if (T == 0) {
    TC_CHECK_CUDA(ctx, cudaMemsetAsync(cb.qoff, 0, sizeof(int64_t) * (TC_NUM_ARMS + 1), ctx->stream));
    TC_CHECK_CUDA(ctx, cudaMemsetAsync(cb.arm_bytes, 0, sizeof(unsigned long long) * TC_NUM_ARMS, ctx->stream));
  } else {
    const size_t plan_smem = opts.selector == TC_SELECT_LEARNED ? TC_MLP_PARAM_COUNT * sizeof(float) : 0;
    PullKeys pk;
    const int64_t K = pull_key_count(g.n, T, ctx->pull_block_tiles, &pk);
    const int64_t per = pk.block_edges / TILE_EDGES, S = (T + per - 1) / per;
    const int64_t slots = PL_INTERLEAVE && S > 1 ? S * per : T;
    const int plan_blocks = (int)((slots + (PLAN_THREADS / 32) - 1) / (PLAN_THREADS / 32));
    TC_CHECK_CUDA(ctx, cudaMemsetAsync(cb.pull_pos, 0, sizeof(uint32_t) * (K + 1), ctx->stream));
    plan_kernel<<<plan_blocks, PLAN_THREADS, plan_smem, ctx->stream>>>(g, T, opts.selector, opts.force_arm,
                                                                       ctx->d_mlp, cb.features, cb.arm, cb.qkeys0,
                                                                       cb.qvals0, cb.tile_bytes, pk, cb.pull_pos, ctx->mlp_margin);
    TC_CHECK_LAUNCH(ctx);
  }
  uint64_t *sk = cb.qkeys0;
  uint32_t *sv = cb.qvals0;
  constexpr int ARM_BITS = 4;  // queue key = (arm << 40) | inverted work
  static_assert(TC_NUM_ARMS <= (1 << ARM_BITS), "arm field of the queue key");
  if (T > 1)
    TC_TRY(radix_sort(ctx, cb.qkeys0, cb.qkeys1, cb.qvals0, cb.qvals1, T, 0, 40 + ARM_BITS, cb.sort_scratch, &sk, &sv));
  if (T > 0) {
    qoff_kernel<<<1, 32, 0, ctx->stream>>>(sk, T, cb.qoff);
    TC_CHECK_LAUNCH(ctx);
    arm_bytes_kernel<<<TC_NUM_ARMS, 256, 0, ctx->stream>>>(sv, cb.qoff, cb.tile_bytes, cb.arm_bytes);
    TC_CHECK_LAUNCH(ctx);
  }
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_heads, 0, sizeof(unsigned) * 64, ctx->stream));
  if (cb.tile_cycles && T > 0)
    TC_CHECK_CUDA(ctx, cudaMemsetAsync(cb.tile_cycles, 0, sizeof(unsigned long long) * T, ctx->stream));
  if (timing) TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[9], ctx->stream));
  for (int a = 0; a < TC_NUM_ARMS; ++a) {
    if (T > 0 && a == TC_ARM_PULL) {
      TC_TRY(run_pull(ctx, g, cb, out, T, timing));
    } else if (T > 0) {
      const int grid = ctx->num_sms * ctx->arm_blocks_per_sm[a];
      arm_kernel(a)<<<grid, arm_threads(a), arm_smem(a), ctx->stream>>>(g, sv, cb.qoff, a, ctx->d_heads + a, out,
                                                                        ctx->d_total, cb.tile_cycles);
      TC_CHECK_LAUNCH(ctx);
    }
    if (timing) TC_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev[10 + a], ctx->stream));
  }
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ctx->h_pinned[PIN_QOFF], cb.qoff, sizeof(int64_t) * (TC_NUM_ARMS + 1),
                                     cudaMemcpyDeviceToHost, ctx->stream));
  TC_CHECK_CUDA(ctx, cudaMemcpyAsync(&ctx->h_pinned[PIN_BYTES], cb.arm_bytes, sizeof(unsigned long long) * TC_NUM_ARMS,
                                     cudaMemcpyDeviceToHost, ctx->stream));
  return TC_OK;
}

static float ev_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return ms;
}

// Triangles through each vertex of the relabelled DAG from the per-edge
// counts c (edge r->s is the lowest pair of c[e] triangles) and the top
// counts (edge r->s joins the lowest and highest vertex of top[e]
// triangles): t[r] += c[e], t[s] += c[e] + top[e]; then per input id.
__global__ void vertex_sum_kernel(DevDag g, const uint32_t *__restrict__ c, const uint32_t *__restrict__ top,
                                  unsigned long long *__restrict__ t) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < g.m; e += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t ce = c[e], te = top[e];
    if (ce) atomicAdd(t + g.src[e], (unsigned long long)ce);
    if (ce + te) atomicAdd(t + g.col[e], (unsigned long long)(ce + te));
  }
}

__global__ void vertex_unrank_kernel(const unsigned long long *__restrict__ t, const int32_t *__restrict__ rank,
                                     int64_t n, unsigned long long *__restrict__ out) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x)
    out[u] = t[rank[u]];
}

__global__ void relabel_u8_kernel(const uint8_t *__restrict__ in, const int32_t *__restrict__ rank, int64_t n,
                                  uint8_t *__restrict__ out) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x)
    out[rank[u]] = in[u];
}

tc_status launch_relabel_u8(tc_ctx *ctx, const uint8_t *in, const int32_t *rank, int64_t n, uint8_t *out) {
  if (n <= 0) return TC_OK;
  relabel_u8_kernel<<<grid_for(ctx, n, 256, 8), 256, 0, ctx->stream>>>(in, rank, n, out);
  TC_CHECK_LAUNCH(ctx);
  return TC_OK;
}

tc_status launch_vertex_sums(tc_ctx *ctx, const DevDag &g, const uint32_t *c, const uint32_t *top,
                             unsigned long long *t, const int32_t *rank, unsigned long long *out) {
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(t, 0, sizeof(unsigned long long) * (size_t)g.n, ctx->stream));
  if (g.m > 0) {
    vertex_sum_kernel<<<grid_for(ctx, g.m, 256, 8), 256, 0, ctx->stream>>>(g, c, top, t);
    TC_CHECK_LAUNCH(ctx);
  }
  vertex_unrank_kernel<<<grid_for(ctx, g.n, 256, 8), 256, 0, ctx->stream>>>(t, rank, g.n, out);
  TC_CHECK_LAUNCH(ctx);
  return TC_OK;
}

// ---- per-partition sums ---------------------------------------------------------
// Each thread folds PS_CHUNK consecutive edges (rows are contiguous, so the
// credited partition rarely changes inside a chunk) and adds each run's sum
// once: into a block-shared table when the partitions fit, else straight
// into the global counters.
constexpr int PS_THREADS = 256;
constexpr int PS_CHUNK = 16;
constexpr int PS_SMEM_PARTS = 4096;

__global__ void part_check_kernel(const int64_t *__restrict__ part, int64_t n, int num_parts, unsigned *flags) {
  bool bad = false;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = part[u];
    bad |= p < 0 || p >= num_parts;
  }
  if (__any_sync(TC_FULL_MASK, bad) && (threadIdx.x & 31) == 0) atomicOr(flags, (unsigned)VF_PART_RANGE);
}

__global__ void __launch_bounds__(PS_THREADS) part_sum_kernel(DevDag g, const uint32_t *__restrict__ c,
                                                              const int64_t *__restrict__ part, int num_parts,
                                                              int rule, unsigned long long *__restrict__ out) {
  extern __shared__ unsigned long long sp[];
  const bool shared_table = num_parts <= PS_SMEM_PARTS;
  if (shared_table)
    for (int q = threadIdx.x; q < num_parts; q += blockDim.x) sp[q] = 0ull;
  __syncthreads();
  unsigned long long *dst = shared_table ? sp : out;
  const int64_t chunks = (g.m + PS_CHUNK - 1) / PS_CHUNK;
  for (int64_t ch = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; ch < chunks;
       ch += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e1 = min(ch * PS_CHUNK + PS_CHUNK, g.m);
    int run = -1;
    unsigned long long acc = 0;
    int32_t u_prev = -1;
    int64_t pu = 0, du = 0;
    for (int64_t e = ch * PS_CHUNK; e < e1; ++e) {
      const uint32_t ce = c[e];
      if (ce == 0) continue;
      const int32_t u = g.src[e];
      if (u != u_prev) {
        u_prev = u;
        pu = part[u];
        du = g.rowptr[u + 1] - g.rowptr[u];
      }
      int64_t p = pu;
      if (rule == TC_PART_PUSH_PULL) {
        const int32_t v = g.col[e];
        const int64_t pv = part[v];
        if (pv != pu && du < g.rowptr[v + 1] - g.rowptr[v]) p = pv;
      }
      if (p < 0 || p >= num_parts) continue;  // flagged by part_check_kernel
      if ((int)p != run) {
        if (run >= 0) atomicAdd(dst + run, acc);
        run = (int)p;
        acc = 0;
      }
      acc += ce;
    }
    if (run >= 0) atomicAdd(dst + run, acc);
  }
  if (shared_table) {
    __syncthreads();
    for (int q = threadIdx.x; q < num_parts; q += blockDim.x)
      if (sp[q]) atomicAdd(out + q, sp[q]);
  }
}

tc_status launch_part_sums(tc_ctx *ctx, const DevDag &g, const uint32_t *c, const int64_t *part, int num_parts,
                           int rule, unsigned long long *out) {
  TC_CHECK_CUDA(ctx, cudaMemsetAsync(out, 0, sizeof(unsigned long long) * (size_t)num_parts, ctx->stream));
  part_check_kernel<<<grid_for(ctx, g.n, 256, 8), 256, 0, ctx->stream>>>(part, g.n, num_parts, ctx->d_flags);
  TC_CHECK_LAUNCH(ctx);
  if (g.m > 0) {
    const size_t smem = num_parts <= PS_SMEM_PARTS ? sizeof(unsigned long long) * (size_t)num_parts : 0;
    part_sum_kernel<<<grid_for(ctx, (g.m + PS_CHUNK - 1) / PS_CHUNK, PS_THREADS, 4), PS_THREADS, smem,
                      ctx->stream>>>(g, c, part, num_parts, rule, out);
    TC_CHECK_LAUNCH(ctx);
  }
  return TC_OK;
}

void count_stats(tc_ctx *ctx, tc_stats *st, bool timing) {
  const int64_t *hq = reinterpret_cast<const int64_t *>(&ctx->h_pinned[PIN_QOFF]);
  const unsigned long long *hb = &ctx->h_pinned[PIN_BYTES];
  uint64_t tot = 0;
  for (int a = 0; a < TC_NUM_ARMS; ++a) {
    st->tiles_per_arm[a] = hq[a + 1] - hq[a];
    st->alg_bytes_arm[a] = hb[a];
    tot += hb[a];
  }
  st->alg_bytes = tot;
  if (!timing) return;
  if (ctx->pull_timed) {
    st->ms_pull_kernel = ev_ms(ctx->ev[10 + TC_NUM_ARMS], ctx->ev[11 + TC_NUM_ARMS]);
    st->pull_edges = (uint64_t)(uint32_t)(ctx->h_pinned[PIN_PULL] & 0xffffffffull);
    ctx->pull_timed = false;
  }
  st->ms_plan = ev_ms(ctx->ev[8], ctx->ev[9]);
  st->ms_count = ev_ms(ctx->ev[9], ctx->ev[10 + TC_NUM_ARMS - 1]);
  for (int a = 0; a < TC_NUM_ARMS; ++a) st->ms_arm[a] = ev_ms(ctx->ev[a == 0 ? 9 : 9 + a], ctx->ev[10 + a]);
}

}  // namespace tc
