// Host half of libtc: seeded generators, the host symmetric-CSR builder,
// GraphMiner file I/O and CSR checks.  C++17 + OpenMP, portable between the
// x86 build container and the Arm (Grace) GPU hosts: no intrinsics.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>
#include <omp.h>

#include "tc_gen_common.h"
#include "tc_internal.h"

namespace tc {

static thread_local char g_err[512] = {0};

void set_global_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
const char *global_error() { return g_err; }

void rmat_thresholds(double a, double b, double c, uint64_t *t1, uint64_t *t2, uint64_t *t3) {
  const double s = 4294967296.0;
  *t1 = (uint64_t)std::floor(a * s);
  *t2 = (uint64_t)std::floor((a + b) * s);
  *t3 = (uint64_t)std::floor((a + b + c) * s);
}

// Expected degrees d_i = C (i+1)^(-1/(gamma-1)) scaled to mean avg_degree,
// capped at sqrt(n * avg_degree) (= sqrt(2m)), stored as 20-bit fixed point
// (at least 1) and accumulated.
void chung_lu_table(int64_t n, double avg_degree, double gamma, uint64_t *cum) {
  const double alpha = 1.0 / (gamma - 1.0);
  std::vector<double> w((size_t)n);
  double sum = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    w[(size_t)i] = std::pow((double)(i + 1), -alpha);
    sum += w[(size_t)i];
  }
  const double scale = avg_degree * (double)n / sum;
  const double cap = std::sqrt((double)n * avg_degree);
  uint64_t acc = 0;
  for (int64_t i = 0; i < n; ++i) {
    double d = std::min(w[(size_t)i] * scale, cap);
    uint64_t fx = (uint64_t)std::llround(d * 1048576.0);
    if (fx == 0) fx = 1;
    acc += fx;
    cum[i] = acc;
  }
}

}  // namespace tc

using namespace tc;

extern "C" {

const char *tc_status_str(tc_status s) {
  switch (s) {
    case TC_OK: return "ok";
    case TC_ERR_INVALID_ARG: return "invalid argument";
    case TC_ERR_INVALID_GRAPH: return "invalid graph";
    case TC_ERR_CUDA: return "CUDA error";
    case TC_ERR_OOM: return "out of memory";
    case TC_ERR_IO: return "I/O error";
    case TC_ERR_TIMEOUT: return "device wait timed out";
    case TC_ERR_UNSUPPORTED: return "unsupported size";
    case TC_ERR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

void tc_opts_default(tc_opts *o) {
  if (!o) return;
  o->selector = TC_SELECT_FIXED;
  o->force_arm = 0;
  o->record_tile_costs = 0;
  o->validate = 1;
}

int64_t tc_gen_num_vertices(const tc_gen_params *p) {
  if (!p) return -1;
  if (p->kind == TC_GEN_RMAT) return (p->scale >= 1 && p->scale <= 30) ? (int64_t(1) << p->scale) : -1;
  return p->n;
}

static tc_status rgg_edges(const tc_gen_params *p, int32_t *src, int32_t *dst, int64_t capacity,
                           int64_t *count_out) {
  const int64_t n = p->n;
  const uint64_t key = tc_stream_key(p->seed, TC_SID_RGG);
  const double r = std::sqrt(p->avg_degree / (M_PI * (double)n));
  const double R = r * 2147483648.0;
  const uint64_t R2 = (uint64_t)std::floor(R * R);
  int64_t cells = (int64_t)std::floor(2147483648.0 / std::max(R, 1.0));
  cells = std::max<int64_t>(1, std::min<int64_t>(cells, 4096));
  const uint64_t side = (2147483648ULL + (uint64_t)cells - 1) / (uint64_t)cells;  // >= R
  std::vector<uint32_t> xs((size_t)n), ys((size_t)n);
  std::vector<int64_t> cell_of((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    tc_rgg_point(key, (uint64_t)i, &xs[(size_t)i], &ys[(size_t)i]);
    const int64_t cx = (int64_t)(xs[(size_t)i] / side), cy = (int64_t)(ys[(size_t)i] / side);
    cell_of[(size_t)i] = cy * cells + cx;
  }
  std::vector<int64_t> cstart((size_t)(cells * cells + 1), 0);
  for (int64_t i = 0; i < n; ++i) cstart[(size_t)cell_of[(size_t)i] + 1]++;
  for (int64_t c = 0; c < cells * cells; ++c) cstart[(size_t)c + 1] += cstart[(size_t)c];
  std::vector<int64_t> cur(cstart.begin(), cstart.end() - 1);
  std::vector<int32_t> order((size_t)n);
  for (int64_t i = 0; i < n; ++i) order[(size_t)cur[(size_t)cell_of[(size_t)i]]++] = (int32_t)i;
  // pass 1 counts, pass 2 writes: pairs (i, j) with i < j within distance.
  std::vector<int64_t> cnt((size_t)n + 1, 0);
  for (int pass = 0; pass < 2; ++pass) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
      const int64_t cx = (int64_t)(xs[(size_t)i] / side), cy = (int64_t)(ys[(size_t)i] / side);
      int64_t k = 0, base = pass ? cnt[(size_t)i] : 0;
      for (int64_t dy = -1; dy <= 1; ++dy) {
        for (int64_t dx = -1; dx <= 1; ++dx) {
          const int64_t nx = cx + dx, ny = cy + dy;
          if (nx < 0 || ny < 0 || nx >= cells || ny >= cells) continue;
          const int64_t c = ny * cells + nx;
          for (int64_t q = cstart[(size_t)c]; q < cstart[(size_t)c + 1]; ++q) {
            const int64_t j = order[(size_t)q];
            if (j <= i) continue;
            const uint64_t ddx = xs[(size_t)i] > xs[(size_t)j] ? xs[(size_t)i] - xs[(size_t)j] : xs[(size_t)j] - xs[(size_t)i];
            const uint64_t ddy = ys[(size_t)i] > ys[(size_t)j] ? ys[(size_t)i] - ys[(size_t)j] : ys[(size_t)j] - ys[(size_t)i];
            if (ddx * ddx + ddy * ddy <= R2) {
              if (pass) { src[base + k] = (int32_t)i; dst[base + k] = (int32_t)j; }
              ++k;
            }
          }
        }
      }
      if (!pass) cnt[(size_t)i] = k;
    }
    if (!pass) {
      int64_t acc = 0;
      for (int64_t i = 0; i < n; ++i) { const int64_t t = cnt[(size_t)i]; cnt[(size_t)i] = acc; acc += t; }
      cnt[(size_t)n] = acc;
      *count_out = acc;
      if (!src || !dst) return TC_OK;  // size query
      if (acc > capacity) {
        set_global_error("RGG produced %lld edges, capacity %lld", (long long)acc, (long long)capacity);
        return TC_ERR_INVALID_ARG;
      }
    }
  }
  return TC_OK;
}

int64_t tc_gen_num_samples(const tc_gen_params *p) {
  if (!p) return -1;
  switch (p->kind) {
    case TC_GEN_ER: return (int64_t)std::floor((double)p->n * p->avg_degree / 2.0);
    case TC_GEN_RMAT: return (int64_t)std::floor(p->edge_factor * (double)(int64_t(1) << p->scale));
    case TC_GEN_CHUNG_LU: return (int64_t)std::floor((double)p->n * p->avg_degree / 2.0);
    case TC_GEN_RGG: {
      int64_t c = 0;
      if (rgg_edges(p, nullptr, nullptr, 0, &c) != TC_OK) return -1;
      return c;
    }
  }
  return -1;
}

static tc_status check_gen(const tc_gen_params *p) {
  if (!p) { set_global_error("null generator params"); return TC_ERR_INVALID_ARG; }
  if (p->kind == TC_GEN_RMAT) {
    if (p->scale < 1 || p->scale > 30) { set_global_error("RMAT scale %d outside [1,30]", p->scale); return TC_ERR_INVALID_ARG; }
    if (!(p->a >= 0 && p->b >= 0 && p->c >= 0 && p->a + p->b + p->c <= 1.0 + 1e-12)) {
      set_global_error("RMAT probabilities must be >= 0 with a+b+c <= 1");
      return TC_ERR_INVALID_ARG;
    }
    if (!(p->edge_factor > 0)) { set_global_error("RMAT edge factor must be > 0"); return TC_ERR_INVALID_ARG; }
    return TC_OK;
  }
  if (p->kind < TC_GEN_ER || p->kind > TC_GEN_CHUNG_LU) { set_global_error("unknown generator %d", p->kind); return TC_ERR_INVALID_ARG; }
  if (p->n < 1 || p->n > 2147483647LL) { set_global_error("n=%lld outside [1, 2^31)", (long long)p->n); return TC_ERR_INVALID_ARG; }
  if (!(p->avg_degree >= 0)) { set_global_error("average degree must be >= 0"); return TC_ERR_INVALID_ARG; }
  if (p->kind == TC_GEN_CHUNG_LU && !(p->gamma > 1.0)) { set_global_error("Chung-Lu gamma must be > 1"); return TC_ERR_INVALID_ARG; }
  return TC_OK;
}

tc_status tc_gen_edges_host(const tc_gen_params *p, int32_t *src, int32_t *dst, int64_t capacity,
                            int64_t *count_out) {
  tc_status st = check_gen(p);
  if (st != TC_OK) return st;
  if (!count_out) { set_global_error("null count_out"); return TC_ERR_INVALID_ARG; }
  if (p->kind == TC_GEN_RGG) return rgg_edges(p, src, dst, capacity, count_out);
  const int64_t M = tc_gen_num_samples(p);
  *count_out = M;
  if (!src || !dst || M > capacity) {
    set_global_error("edge buffers hold %lld samples, %lld needed", (long long)capacity, (long long)M);
    return TC_ERR_INVALID_ARG;
  }
  if (p->kind == TC_GEN_ER) {
    const uint64_t key = tc_stream_key(p->seed, TC_SID_ER);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < M; ++i) tc_er_sample(key, (uint64_t)p->n, (uint64_t)i, &src[i], &dst[i]);
  } else if (p->kind == TC_GEN_RMAT) {
    const uint64_t key = tc_stream_key(p->seed, TC_SID_RMAT);
    uint64_t t1, t2, t3;
    rmat_thresholds(p->a, p->b, p->c, &t1, &t2, &t3);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < M; ++i) tc_rmat_sample(key, p->scale, t1, t2, t3, (uint64_t)i, &src[i], &dst[i]);
  } else {
    const uint64_t key = tc_stream_key(p->seed, TC_SID_CL);
    std::vector<uint64_t> cum((size_t)p->n);
    chung_lu_table(p->n, p->avg_degree, p->gamma, cum.data());
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < M; ++i) tc_cl_sample(key, cum.data(), p->n, (uint64_t)i, &src[i], &dst[i]);
  }
  return TC_OK;
}

tc_status tc_csr_from_edges_host(int64_t n, int64_t num_edges, const int32_t *src, const int32_t *dst,
                                 int64_t **rowptr_out, int32_t **colidx_out, int64_t *nnz_out) {
  if (n < 1 || n > 2147483647LL || num_edges < 0 || (num_edges > 0 && (!src || !dst)) || !rowptr_out ||
      !colidx_out || !nnz_out) {
    set_global_error("tc_csr_from_edges_host: bad arguments");
    return TC_ERR_INVALID_ARG;
  }
  for (int64_t i = 0; i < num_edges; ++i) {
    if (src[i] < 0 || src[i] >= n || dst[i] < 0 || dst[i] >= n) {
      set_global_error("edge %lld (%d,%d) has an id outside [0,%lld)", (long long)i, src[i], dst[i], (long long)n);
      return TC_ERR_INVALID_GRAPH;
    }
  }
  std::vector<int64_t> deg((size_t)n + 1, 0);
  for (int64_t i = 0; i < num_edges; ++i) {
    if (src[i] == dst[i]) continue;
    deg[(size_t)src[i]]++;
    deg[(size_t)dst[i]]++;
  }
  std::vector<int64_t> off((size_t)n + 1, 0);
  for (int64_t u = 0; u < n; ++u) off[(size_t)u + 1] = off[(size_t)u] + deg[(size_t)u];
  std::vector<int32_t> tmp((size_t)off[(size_t)n]);
  std::vector<int64_t> cur(off.begin(), off.end() - 1);
  for (int64_t i = 0; i < num_edges; ++i) {
    if (src[i] == dst[i]) continue;
    tmp[(size_t)cur[(size_t)src[i]]++] = dst[i];
    tmp[(size_t)cur[(size_t)dst[i]]++] = src[i];
  }
  std::vector<int64_t> ndeg((size_t)n, 0);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t u = 0; u < n; ++u) {
    int32_t *b = tmp.data() + off[(size_t)u], *e = tmp.data() + off[(size_t)u + 1];
    std::sort(b, e);
    ndeg[(size_t)u] = std::unique(b, e) - b;
  }
  int64_t *rowptr = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
  if (!rowptr) { set_global_error("host allocation failed"); return TC_ERR_OOM; }
  rowptr[0] = 0;
  for (int64_t u = 0; u < n; ++u) rowptr[u + 1] = rowptr[u] + ndeg[(size_t)u];
  const int64_t nnz = rowptr[n];
  int32_t *col = (int32_t *)malloc(sizeof(int32_t) * (size_t)std::max<int64_t>(nnz, 1));
  if (!col) { free(rowptr); set_global_error("host allocation failed"); return TC_ERR_OOM; }
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t u = 0; u < n; ++u)
    std::copy(tmp.data() + off[(size_t)u], tmp.data() + off[(size_t)u] + ndeg[(size_t)u], col + rowptr[u]);
  *rowptr_out = rowptr;
  *colidx_out = col;
  *nnz_out = nnz;
  return TC_OK;
}

// Sequential symmetric CSR of one small graph (used per graph, in parallel
// over graphs).
static void local_csr(int64_t n, const std::vector<int32_t> &src, const std::vector<int32_t> &dst,
                      std::vector<int64_t> &rowptr, std::vector<int32_t> &col) {
  std::vector<int64_t> off((size_t)n + 1, 0);
  for (size_t i = 0; i < src.size(); ++i) {
    if (src[i] == dst[i]) continue;
    off[(size_t)src[i] + 1]++;
    off[(size_t)dst[i] + 1]++;
  }
  for (int64_t v = 0; v < n; ++v) off[(size_t)v + 1] += off[(size_t)v];
  std::vector<int32_t> tmp((size_t)off[(size_t)n]);
  std::vector<int64_t> cur(off.begin(), off.end() - 1);
  for (size_t i = 0; i < src.size(); ++i) {
    if (src[i] == dst[i]) continue;
    tmp[(size_t)cur[(size_t)src[i]]++] = dst[i];
    tmp[(size_t)cur[(size_t)dst[i]]++] = src[i];
  }
  rowptr.assign((size_t)n + 1, 0);
  col.clear();
  col.reserve(tmp.size());
  for (int64_t v = 0; v < n; ++v) {
    int32_t *b = tmp.data() + off[(size_t)v], *e = tmp.data() + off[(size_t)v + 1];
    std::sort(b, e);
    e = std::unique(b, e);
    col.insert(col.end(), b, e);
    rowptr[(size_t)v + 1] = (int64_t)col.size();
  }
}

tc_status tc_gen_batch_host(const tc_batch_spec *spec, int64_t *vtx_off, int64_t **rowptr_out, int32_t **colidx_out,
                            int64_t *nnz_out) {
  if (!spec || !vtx_off || !rowptr_out || !colidx_out || !nnz_out || spec->num_graphs < 1 || spec->n_min < 2 ||
      spec->n_max < spec->n_min || spec->n_max > (int64_t(1) << 24) || !(spec->deg_min >= 0) ||
      !(spec->deg_max >= spec->deg_min)) {
    set_global_error("tc_gen_batch_host: bad spec");
    return TC_ERR_INVALID_ARG;
  }
  const int64_t G = spec->num_graphs;
  std::vector<std::vector<int64_t>> rows((size_t)G);
  std::vector<std::vector<int32_t>> cols((size_t)G);
  std::vector<int64_t> nv((size_t)G);
  int failed = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(max : failed)
  for (int64_t g = 0; g < G; ++g) {
    const uint64_t sg = tc_mix64(spec->seed * 0x9E3779B97F4A7C15ULL + (uint64_t)g + 1);
    const uint64_t key = tc_stream_key(sg, 5);
    const double u1 = (double)(tc_rand_at(key, 0) >> 11) * (1.0 / 9007199254740992.0);
    const double u2 = (double)(tc_rand_at(key, 1) >> 11) * (1.0 / 9007199254740992.0);
    int64_t n = (int64_t)std::llround(std::exp(std::log((double)spec->n_min) +
                                               u1 * (std::log((double)spec->n_max) - std::log((double)spec->n_min))));
    const double deg = spec->deg_min + u2 * (spec->deg_max - spec->deg_min);
    tc_gen_params p;
    memset(&p, 0, sizeof(p));
    p.seed = sg;
    p.avg_degree = deg;
    p.a = spec->a;
    p.b = spec->b;
    p.c = spec->c;
    switch (g % 3) {
      case 0: p.kind = TC_GEN_ER; p.n = n; break;
      case 1: {
        p.kind = TC_GEN_RMAT;
        p.scale = std::max(1, (int)std::lround(std::log2((double)n)));
        p.edge_factor = deg / 2.0;
        n = int64_t(1) << p.scale;
        break;
      }
      default: p.kind = TC_GEN_RGG; p.n = n; break;
    }
    const int64_t cap = tc_gen_num_samples(&p);
    std::vector<int32_t> s((size_t)std::max<int64_t>(cap, 1)), d((size_t)std::max<int64_t>(cap, 1));
    int64_t cnt = 0;
    if (cap < 0 || tc_gen_edges_host(&p, s.data(), d.data(), cap, &cnt) != TC_OK) {
      failed = 1;
      continue;
    }
    s.resize((size_t)cnt);
    d.resize((size_t)cnt);
    nv[(size_t)g] = n;
    local_csr(n, s, d, rows[(size_t)g], cols[(size_t)g]);
  }
  if (failed) {
    set_global_error("tc_gen_batch_host: a graph failed to generate");
    return TC_ERR_INVALID_ARG;
  }
  vtx_off[0] = 0;
  int64_t nnz = 0;
  for (int64_t g = 0; g < G; ++g) {
    vtx_off[g + 1] = vtx_off[g] + nv[(size_t)g];
    nnz += (int64_t)cols[(size_t)g].size();
  }
  const int64_t N = vtx_off[G];
  if (N > 2147483647LL) {
    set_global_error("batch holds %lld vertices", (long long)N);
    return TC_ERR_UNSUPPORTED;
  }
  int64_t *rowptr = (int64_t *)malloc(sizeof(int64_t) * (size_t)(N + 1));
  int32_t *col = (int32_t *)malloc(sizeof(int32_t) * (size_t)std::max<int64_t>(nnz, 1));
  if (!rowptr || !col) {
    free(rowptr);
    free(col);
    set_global_error("host allocation failed");
    return TC_ERR_OOM;
  }
  std::vector<int64_t> ebase((size_t)G + 1, 0);
  for (int64_t g = 0; g < G; ++g) ebase[(size_t)g + 1] = ebase[(size_t)g] + (int64_t)cols[(size_t)g].size();
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t g = 0; g < G; ++g) {
    const std::vector<int64_t> &r = rows[(size_t)g];
    for (int64_t v = 0; v < nv[(size_t)g]; ++v) rowptr[vtx_off[g] + v] = ebase[(size_t)g] + r[(size_t)v];
    std::copy(cols[(size_t)g].begin(), cols[(size_t)g].end(), col + ebase[(size_t)g]);
  }
  rowptr[N] = nnz;
  *rowptr_out = rowptr;
  *colidx_out = col;
  *nnz_out = nnz;
  return TC_OK;
}

tc_status tc_check_csr_host(int64_t n, int64_t nnz, const int64_t *rowptr, const int32_t *colidx,
                            int32_t require_sorted_simple) {
  if (n < 0 || nnz < 0 || !rowptr || (nnz > 0 && !colidx)) {
    set_global_error("tc_check_csr_host: bad arguments");
    return TC_ERR_INVALID_ARG;
  }
  if (rowptr[0] != 0 || rowptr[n] != nnz) {
    set_global_error("rowptr[0]=%lld rowptr[n]=%lld, expected 0 and nnz=%lld", (long long)rowptr[0],
                     (long long)rowptr[n], (long long)nnz);
    return TC_ERR_INVALID_GRAPH;
  }
  int bad = 0;
  int64_t bad_at = -1;
#pragma omp parallel for schedule(dynamic, 4096) reduction(max : bad)
  for (int64_t u = 0; u < n; ++u) {
    if (rowptr[u + 1] < rowptr[u]) { bad = std::max(bad, 1); continue; }
    for (int64_t e = rowptr[u]; e < rowptr[u + 1]; ++e) {
      const int32_t v = colidx[e];
      if (v < 0 || v >= n) { bad = std::max(bad, 2); break; }
      if (require_sorted_simple) {
        if (v == u) { bad = std::max(bad, 3); break; }
        if (e > rowptr[u] && colidx[e - 1] >= v) { bad = std::max(bad, 4); break; }
      }
    }
  }
  (void)bad_at;
  static const char *why[] = {"", "rowptr is not monotone", "a column id is outside [0, n)",
                              "a row holds a self loop", "a row is not strictly ascending"};
  if (bad) { set_global_error("%s", why[bad]); return TC_ERR_INVALID_GRAPH; }
  return TC_OK;
}

// ---- GraphMiner files ------------------------------------------------------

static bool read_exact(const std::string &path, void *buf, size_t bytes) {
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) return false;
  size_t got = bytes ? fread(buf, 1, bytes, f) : 0;
  bool ok = got == bytes;
  if (ok) {  // no trailing bytes either: a longer file is a different graph
    char extra;
    ok = fread(&extra, 1, 1, f) == 0;
  }
  fclose(f);
  return ok;
}

tc_status tc_load_graphminer(const char *prefix, int64_t *n_out, int64_t *nnz_out, int64_t **rowptr_out,
                             int32_t **colidx_out, int64_t *max_degree_out) {
  if (!prefix || !n_out || !nnz_out || !rowptr_out || !colidx_out) {
    set_global_error("tc_load_graphminer: null argument");
    return TC_ERR_INVALID_ARG;
  }
  const std::string p(prefix);
  std::ifstream meta((p + ".meta.txt").c_str());
  if (!meta) { set_global_error("cannot open %s.meta.txt", prefix); return TC_ERR_IO; }
  long long n = 0, nnz = 0, vid_size = 0, eid_size = 0, vl = 0, el = 0, maxd = 0, feat = 0, nvc = 0, nec = 0;
  meta >> n >> nnz >> vid_size >> eid_size >> vl >> el >> maxd >> feat >> nvc >> nec;
  if (!meta) { set_global_error("%s.meta.txt: expected 10 integers", prefix); return TC_ERR_IO; }
  if (vid_size != 4 || eid_size != 8) {
    set_global_error("%s.meta.txt: vid_size=%lld eid_size=%lld, this engine reads 4 and 8", prefix, vid_size, eid_size);
    return TC_ERR_UNSUPPORTED;
  }
  if (n < 1 || n > 2147483647LL || nnz < 0) { set_global_error("%s.meta.txt: bad sizes", prefix); return TC_ERR_IO; }
  int64_t *rowptr = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
  int32_t *col = (int32_t *)malloc(sizeof(int32_t) * (size_t)std::max<long long>(nnz, 1));
  if (!rowptr || !col) { free(rowptr); free(col); set_global_error("host allocation failed"); return TC_ERR_OOM; }
  if (!read_exact(p + ".vertex.bin", rowptr, sizeof(int64_t) * (size_t)(n + 1)) ||
      !read_exact(p + ".edge.bin", col, sizeof(int32_t) * (size_t)nnz)) {
    free(rowptr); free(col);
    set_global_error("%s.vertex.bin / .edge.bin missing or of the wrong length", prefix);
    return TC_ERR_IO;
  }
  tc_status st = tc_check_csr_host(n, nnz, rowptr, col, 0);
  if (st != TC_OK) { free(rowptr); free(col); return st; }
  *n_out = n;
  *nnz_out = nnz;
  *rowptr_out = rowptr;
  *colidx_out = col;
  if (max_degree_out) *max_degree_out = maxd;
  return TC_OK;
}

tc_status tc_save_graphminer(const char *prefix, int64_t n, int64_t nnz, const int64_t *rowptr,
                             const int32_t *colidx) {
  if (!prefix || n < 1 || nnz < 0 || !rowptr || (nnz > 0 && !colidx)) {
    set_global_error("tc_save_graphminer: bad arguments");
    return TC_ERR_INVALID_ARG;
  }
  tc_status st = tc_check_csr_host(n, nnz, rowptr, colidx, 0);
  if (st != TC_OK) return st;
  int64_t maxd = 0;
  for (int64_t u = 0; u < n; ++u) maxd = std::max<int64_t>(maxd, rowptr[u + 1] - rowptr[u]);
  const std::string p(prefix);
  FILE *f = fopen((p + ".meta.txt").c_str(), "w");
  if (!f) { set_global_error("cannot write %s.meta.txt", prefix); return TC_ERR_IO; }
  fprintf(f, "%lld\n%lld\n4 8 1 4\n%lld\n0\n0\n0\n", (long long)n, (long long)nnz, (long long)maxd);
  fclose(f);
  f = fopen((p + ".vertex.bin").c_str(), "wb");
  if (!f) { set_global_error("cannot write %s.vertex.bin", prefix); return TC_ERR_IO; }
  bool ok = fwrite(rowptr, sizeof(int64_t), (size_t)(n + 1), f) == (size_t)(n + 1);
  fclose(f);
  f = fopen((p + ".edge.bin").c_str(), "wb");
  if (!f) { set_global_error("cannot write %s.edge.bin", prefix); return TC_ERR_IO; }
  ok = ok && (nnz == 0 || fwrite(colidx, sizeof(int32_t), (size_t)nnz, f) == (size_t)nnz);
  fclose(f);
  if (!ok) { set_global_error("short write under %s", prefix); return TC_ERR_IO; }
  return TC_OK;
}

// ---- METIS partition files (read-only) --------------------------------------

void tc_metis_part_free(tc_metis_part *p) {
  if (!p) return;
  free(p->rowptr);
  free(p->colidx);
  free(p->vertex_list);
  free(p->part);
  p->rowptr = nullptr;
  p->colidx = nullptr;
  p->vertex_list = nullptr;
  p->part = nullptr;
}

void tc_host_free(void *p) { free(p); }

tc_status tc_load_metis_part(const char *prefix, tc_metis_part *out) {
  if (!prefix || !out) {
    set_global_error("tc_load_metis_part: null argument");
    return TC_ERR_INVALID_ARG;
  }
  memset(out, 0, sizeof(*out));
  const std::string p(prefix);
  std::ifstream meta((p + ".meta.txt").c_str());
  if (!meta) { set_global_error("cannot open %s.meta.txt", prefix); return TC_ERR_IO; }
  long long v[6] = {0, 0, 0, 0, 0, 0};
  for (long long &x : v) meta >> x;
  if (!meta) { set_global_error("%s.meta.txt: expected 6 integers", prefix); return TC_ERR_IO; }
  const long long n = v[0], n_real = v[1], nnz = v[2];
  if (n < 1 || n > 2147483647LL || n_real < 0 || n_real > n || nnz < 0) {
    set_global_error("%s.meta.txt: bad sizes n=%lld n_real=%lld nnz=%lld", prefix, n, n_real, nnz);
    return TC_ERR_IO;
  }
  tc_metis_part r;
  r.n = n;
  r.n_real = n_real;
  r.nnz = nnz;
  r.max_subg_nv = v[3];
  r.max_subg_ne = v[4];
  r.max_degree = v[5];
  r.rowptr = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
  r.colidx = (int32_t *)malloc(sizeof(int32_t) * (size_t)std::max<long long>(nnz, 1));
  r.vertex_list = (int32_t *)malloc(sizeof(int32_t) * (size_t)std::max<long long>(n_real, 1));
  r.part = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
  if (!r.rowptr || !r.colidx || !r.vertex_list || !r.part) {
    tc_metis_part_free(&r);
    set_global_error("host allocation failed");
    return TC_ERR_OOM;
  }
  if (!read_exact(p + ".vertex.bin", r.rowptr, sizeof(int64_t) * (size_t)(n + 1)) ||
      !read_exact(p + ".edge.bin", r.colidx, sizeof(int32_t) * (size_t)nnz) ||
      !read_exact(p + ".vertex_list.bin", r.vertex_list, sizeof(int32_t) * (size_t)n_real) ||
      !read_exact(p + ".part.bin", r.part, sizeof(int64_t) * (size_t)n)) {
    tc_metis_part_free(&r);
    set_global_error("%s: .vertex.bin / .edge.bin / .vertex_list.bin / .part.bin missing or of the wrong length",
                     prefix);
    return TC_ERR_IO;
  }
  tc_status st = tc_check_csr_host(n, nnz, r.rowptr, r.colidx, 0);
  if (st != TC_OK) { tc_metis_part_free(&r); return st; }
  for (long long i = 0; i < n_real; ++i) {
    if (r.vertex_list[i] < 0 || r.vertex_list[i] >= n) {
      tc_metis_part_free(&r);
      set_global_error("%s.vertex_list.bin: vertex %d outside [0, %lld)", prefix, (int)r.vertex_list[i], n);
      return TC_ERR_INVALID_GRAPH;
    }
  }
  *out = r;
  return TC_OK;
}

// Two passes over the file sets, one set in memory at a time: the first
// checks every set and records the lengths of its own rows, the second
// copies those rows.  Memory: the part table, the result and one set.
tc_status tc_assemble_metis(const char *prefix, int32_t num_parts, int64_t *n_out, int64_t *nnz_out,
                            int64_t **rowptr_out, int32_t **colidx_out, int64_t **part_out) {
  if (!prefix || num_parts < 1 || !n_out || !nnz_out || !rowptr_out || !colidx_out) {
    set_global_error("tc_assemble_metis: bad arguments");
    return TC_ERR_INVALID_ARG;
  }
  auto name = [&](int32_t k) { return std::string(prefix) + std::to_string(k); };
  tc_metis_part q;
  memset(&q, 0, sizeof(q));
  std::vector<int64_t> part, len, owned;
  int64_t n = 0;
  tc_status st = TC_OK;
  for (int32_t k = 0; k < num_parts && st == TC_OK; ++k) {  // pass 1: checks and row lengths
    st = tc_load_metis_part(name(k).c_str(), &q);
    if (st != TC_OK) break;
    if (k == 0) {
      n = q.n;
      part.assign(q.part, q.part + n);
      len.assign((size_t)n, 0);
      owned.assign((size_t)num_parts, 0);
      for (int64_t v = 0; v < n; ++v) {
        if (part[(size_t)v] < 0 || part[(size_t)v] >= num_parts) {
          set_global_error("%s0.part.bin: vertex %lld in partition %lld, outside [0, %d)", prefix, (long long)v,
                           (long long)part[(size_t)v], (int)num_parts);
          st = TC_ERR_INVALID_GRAPH;
          break;
        }
        ++owned[(size_t)part[(size_t)v]];
      }
    } else if (q.n != n || memcmp(q.part, part.data(), sizeof(int64_t) * (size_t)n) != 0) {
      set_global_error("%s%d: vertex count or part table differs from %s0", prefix, (int)k, prefix);
      st = TC_ERR_INVALID_GRAPH;
    }
    if (st == TC_OK && q.n_real != owned[(size_t)k]) {
      set_global_error("%s%d.vertex_list.bin lists %lld vertices, the part table gives partition %d %lld", prefix,
                       (int)k, (long long)q.n_real, (int)k, (long long)owned[(size_t)k]);
      st = TC_ERR_INVALID_GRAPH;
    }
    int64_t own_entries = 0;
    for (int64_t i = 0; st == TC_OK && i < q.n_real; ++i) {
      const int64_t v = q.vertex_list[i];
      if (part[(size_t)v] != k || (i > 0 && q.vertex_list[i - 1] >= v)) {
        set_global_error("%s%d.vertex_list.bin does not list partition %d's vertices in order (entry %lld)", prefix,
                         (int)k, (int)k, (long long)i);
        st = TC_ERR_INVALID_GRAPH;
        break;
      }
      len[(size_t)v] = q.rowptr[v + 1] - q.rowptr[v];
      own_entries += len[(size_t)v];
    }
    // rows are monotone, so the own rows hold every entry exactly when all
    // other rows are empty
    if (st == TC_OK && own_entries != q.nnz) {
      set_global_error("%s%d: rows of vertices outside partition %d hold entries", prefix, (int)k, (int)k);
      st = TC_ERR_INVALID_GRAPH;
    }
    tc_metis_part_free(&q);
  }
  if (st != TC_OK) return st;
  int64_t *rowptr = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
  if (!rowptr) { set_global_error("host allocation failed"); return TC_ERR_OOM; }
  rowptr[0] = 0;
  for (int64_t v = 0; v < n; ++v) rowptr[v + 1] = rowptr[v] + len[(size_t)v];
  const int64_t nnz = rowptr[n];
  int32_t *col = (int32_t *)malloc(sizeof(int32_t) * (size_t)std::max<int64_t>(nnz, 1));
  int64_t *part_copy = part_out ? (int64_t *)malloc(sizeof(int64_t) * (size_t)n) : nullptr;
  if (!col || (part_out && !part_copy)) {
    free(rowptr); free(col); free(part_copy);
    set_global_error("host allocation failed");
    return TC_ERR_OOM;
  }
  for (int32_t k = 0; k < num_parts && st == TC_OK; ++k) {  // pass 2: the own rows' columns
    st = tc_load_metis_part(name(k).c_str(), &q);
    if (st != TC_OK) break;
    if (q.n != n || q.n_real != owned[(size_t)k]) {  // the file set changed between the passes
      set_global_error("%s%d changed while it was read", prefix, (int)k);
      st = TC_ERR_IO;
    }
    for (int64_t i = 0; st == TC_OK && i < q.n_real; ++i) {
      const int64_t v = q.vertex_list[i];
      if (v < 0 || v >= n || part[(size_t)v] != k || q.rowptr[v + 1] - q.rowptr[v] != len[(size_t)v]) {
        set_global_error("%s%d changed while it was read", prefix, (int)k);
        st = TC_ERR_IO;
        break;
      }
      memcpy(col + rowptr[v], q.colidx + q.rowptr[v], sizeof(int32_t) * (size_t)len[(size_t)v]);
    }
    tc_metis_part_free(&q);
  }
  if (st != TC_OK) {
    free(rowptr); free(col); free(part_copy);
    return st;
  }
  if (part_copy) memcpy(part_copy, part.data(), sizeof(int64_t) * (size_t)n);
  *n_out = n;
  *nnz_out = nnz;
  *rowptr_out = rowptr;
  *colidx_out = col;
  if (part_out) *part_out = part_copy;
  return TC_OK;
}

tc_status tc_load_vlabels(const char *prefix, int64_t n, uint8_t *labels) {
  if (!prefix || n < 1 || !labels) {
    set_global_error("tc_load_vlabels: bad arguments");
    return TC_ERR_INVALID_ARG;
  }
  if (!read_exact(std::string(prefix) + ".vlabel.bin", labels, (size_t)n)) {
    set_global_error("%s.vlabel.bin missing or not %lld bytes", prefix, (long long)n);
    return TC_ERR_IO;
  }
  return TC_OK;
}

tc_status tc_save_vlabels(const char *prefix, int64_t n, const uint8_t *labels) {
  if (!prefix || n < 1 || !labels) {
    set_global_error("tc_save_vlabels: bad arguments");
    return TC_ERR_INVALID_ARG;
  }
  const std::string p(prefix);
  long long v[10] = {0};
  {
    std::ifstream meta((p + ".meta.txt").c_str());
    if (!meta) { set_global_error("cannot open %s.meta.txt (save the graph first)", prefix); return TC_ERR_IO; }
    for (int i = 0; i < 10; ++i) meta >> v[i];
    if (!meta) { set_global_error("%s.meta.txt: expected 10 integers", prefix); return TC_ERR_IO; }
  }
  if (v[0] != n) { set_global_error("%s.meta.txt holds n=%lld, not %lld", prefix, v[0], (long long)n); return TC_ERR_INVALID_ARG; }
  int maxl = 0;
  for (int64_t u = 0; u < n; ++u) maxl = std::max<int>(maxl, labels[u]);
  v[4] = 1;         // vlabel_size: one byte per vertex
  v[8] = maxl + 1;  // num_vertex_classes
  FILE *f = fopen((p + ".meta.txt").c_str(), "w");
  if (!f) { set_global_error("cannot write %s.meta.txt", prefix); return TC_ERR_IO; }
  fprintf(f, "%lld\n%lld\n%lld %lld %lld %lld\n%lld\n%lld\n%lld\n%lld\n", v[0], v[1], v[2], v[3], v[4], v[5], v[6],
          v[7], v[8], v[9]);
  fclose(f);
  f = fopen((p + ".vlabel.bin").c_str(), "wb");
  if (!f) { set_global_error("cannot write %s.vlabel.bin", prefix); return TC_ERR_IO; }
  const bool ok = fwrite(labels, 1, (size_t)n, f) == (size_t)n;
  fclose(f);
  if (!ok) { set_global_error("short write of %s.vlabel.bin", prefix); return TC_ERR_IO; }
  return TC_OK;
}

void tc_csr_free(int64_t *rowptr, int32_t *colidx) {
  free(rowptr);
  free(colidx);
}

}  // extern "C"
