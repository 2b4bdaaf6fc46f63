// Allocation-free triangle count of an oriented graph.
//
// Some callers cannot allocate device memory on the counting path: programs
// whose runtime owns the whole device through its own memory pool (a serving
// stack that pre-reserves the GPU and forbids cudaMalloc outside the pool),
// plugins loaded into such a host, and latency-bound loops where cudaMalloc's
// implicit device synchronisation is not acceptable.  tc_count_dag_noalloc
// serves them: it is a variant of the HASH count kernel (count.cu) whose
// scratch — the work counter and the first row of every 512-edge work item —
// lives in the fixed, file-scope device array below instead of the ctx arena.
// It allocates nothing and creates no ctx; every GPU that loads the library
// holds the array (TC_NOALLOC_SCRATCH_BYTES) until the process exits.
//
// The array is shared by every call: a call overwrites what the previous one
// left, and the kernels clear the counter they need before use.  Calls whose
// kernels overlap on the GPU (different streams or host threads without
// ordering) race on the array and give wrong results.
#include <algorithm>
#include <mutex>

#include <cuda.h>

#include "engine.cuh"

namespace tc {

constexpr int NA_THREADS = 256;
constexpr int NA_WARPS = NA_THREADS / 32;
constexpr int NA_ITEM = 512;                    // edges per warp work item
constexpr int NA_SLOTS = 1024;                  // per-warp hash table
constexpr int64_t NA_HEADER = 256;              // bytes before the item-row table
constexpr int64_t NA_MAX_ITEMS = ((int64_t)TC_NOALLOC_SCRATCH_BYTES - NA_HEADER) / 4;

static __device__ __align__(256) unsigned char g_noalloc_scratch[TC_NOALLOC_SCRATCH_BYTES];

// Header: [0] work counter (uint32).  Then int32 item_row[items].
__global__ void noalloc_prep_kernel(const int64_t *__restrict__ rowptr, int64_t n, int64_t m, int64_t items,
                                    unsigned char *scratch, unsigned long long *total) {
  unsigned *head = reinterpret_cast<unsigned *>(scratch);
  int32_t *item_row = reinterpret_cast<int32_t *>(scratch + NA_HEADER);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < items; i += (int64_t)gridDim.x * blockDim.x)
    item_row[i] = (int32_t)row_of_entry(rowptr, n, i * NA_ITEM);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *head = 0u;
    *total = 0ull;
  }
}

__device__ __forceinline__ uint32_t na_slot(int32_t x, int bits) { return ((uint32_t)x * 0x9E3779B1u) >> (32 - bits); }

__global__ void __launch_bounds__(NA_THREADS) noalloc_hash_kernel(const int64_t *__restrict__ rowptr,
                                                                 const int32_t *__restrict__ col, int64_t n,
                                                                 int64_t m, int64_t items, unsigned char *scratch,
                                                                 unsigned long long *total, uint32_t *out) {
  __shared__ int32_t tab[NA_WARPS][NA_SLOTS];
  __shared__ int32_t s_incl[NA_WARPS][32];
  __shared__ long long s_base[NA_WARPS][32];
  __shared__ uint32_t s_hits[NA_WARPS][32];
  unsigned *head = reinterpret_cast<unsigned *>(scratch);
  const int32_t *item_row = reinterpret_cast<const int32_t *>(scratch + NA_HEADER);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t *T = tab[w];
  unsigned long long acc = 0;
  for (;;) {
    unsigned it = 0;
    if (lane == 0) it = atomicAdd(head, 1u);
    it = __shfl_sync(TC_FULL_MASK, it, 0);
    if ((int64_t)it >= items) break;
    const int64_t e0 = (int64_t)it * NA_ITEM, e1 = min(m, e0 + NA_ITEM);
    int64_t r = item_row[it];
    for (int64_t e = e0; e < e1;) {
      while (rowptr[r + 1] <= e) ++r;  // skip rows that end before e (empty rows included)
      const int64_t rb = rowptr[r], re = rowptr[r + 1];
      const int64_t se = min(e1, re);
      const int na = (int)(re - rb);
      if (na > NA_SLOTS / 2) {  // long row: warp binary search per edge
        for (int64_t k = e; k < se; ++k) {
          const int32_t s = col[k];
          uint32_t c = 0;
          if (s >= 0 && (int64_t)s < n) {
            const int32_t *B = col + rowptr[s];
            const int nb = (int)(rowptr[s + 1] - rowptr[s]);
            const int32_t *A = col + rb;
            const int32_t *L = na <= nb ? A : B, *S = na <= nb ? B : A;
            const int nl = na <= nb ? na : nb, ns = na <= nb ? nb : na;
            int lo = 0;
            for (int i = lane; i < nl; i += 32) {
              const int32_t key = L[i];
              int hi = ns;
              while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (S[mid] < key) lo = mid + 1; else hi = mid;
              }
              if (lo < ns && S[lo] == key) ++c;
            }
          }
          c = warp_sum(c);
          if (lane == 0) {
            if (out) out[k] = c;
            acc += c;
          }
        }
        e = se;
        continue;
      }
      int bits = 5;
      while ((1 << bits) < 2 * na) ++bits;
      const uint32_t mask = (1u << bits) - 1u;
      for (int k = lane; k < (1 << bits); k += 32) T[k] = -1;
      __syncwarp();
      for (int k = lane; k < na; k += 32) {
        const int32_t x = col[rb + k];
        uint32_t sl = na_slot(x, bits);
        while (atomicCAS(&T[sl], -1, x) != -1) sl = (sl + 1) & mask;
      }
      __syncwarp();
      for (int64_t eb = e; eb < se; eb += 32) {
        const int64_t ei = eb + lane;
        int nb = 0;
        long long bst = 0;
        if (ei < se) {
          const int32_t s = col[ei];
          if (s >= 0 && (int64_t)s < n) {
            bst = rowptr[s];
            nb = (int)(rowptr[s + 1] - bst);
          }
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
          const int32_t x = col[cur_base + p];
          uint32_t sl = na_slot(x, bits);
          for (;;) {
            const int32_t v = T[sl];
            if (v == x) { atomicAdd(&s_hits[w][i], 1u); break; }
            if (v == -1) break;
            sl = (sl + 1) & mask;
          }
        }
        __syncwarp();
        if (ei < se) {
          const uint32_t c = s_hits[w][lane];
          if (out) out[ei] = c;
          acc += c;
        }
        __syncwarp();
      }
      e = se;
      __syncwarp();
    }
  }
  acc = warp_sum(acc);
  if (lane == 0 && acc) atomicAdd(total, acc);
}

static std::mutex g_na_mu;
static void *g_na_ptr[64] = {};
static unsigned long long g_na_ctx[64] = {};  // context the cached address belongs to

// Identity of the calling thread's current context (unique for the life of
// the process, so a context created after cudaDeviceReset gets a new one);
// 0 when the driver does not report it.  The driver calls are reached through
// the runtime's entry-point query, so the library does not link libcuda.
static unsigned long long current_ctx_id() {
  typedef CUresult (*GetCurrent)(CUcontext *);
  typedef CUresult (*GetId)(CUcontext, unsigned long long *);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool resolved = false;
  if (!resolved) {
    void *a = nullptr, *b = nullptr;
    cudaDriverEntryPointQueryResult qa, qb;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
        qa == cudaDriverEntryPointSuccess && qb == cudaDriverEntryPointSuccess) {
      get_current = (GetCurrent)a;
      get_id = (GetId)b;
    }
    (void)cudaGetLastError();
    resolved = true;
  }
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&c) == CUDA_SUCCESS && c && get_id(c, &id) == CUDA_SUCCESS) return id;
  return 0;
}

}  // namespace tc

using namespace tc;

extern "C" tc_status tc_count_dag_noalloc(int device, const int64_t *rowptr, const int32_t *colidx, int64_t n,
                                          int64_t m, uint64_t *total, uint32_t *edge_counts, void *stream) {
  if (device < 0 || device >= 64) return set_error(nullptr, TC_ERR_INVALID_ARG, "device %d outside [0,64)", device);
  if (!rowptr || !total || (m > 0 && !colidx) || n < 1 || n > 2147483647LL || m < 0)
    return set_error(nullptr, TC_ERR_INVALID_ARG, "tc_count_dag_noalloc: null pointer or bad n/m");
  const int64_t items = (m + NA_ITEM - 1) / NA_ITEM;
  if (items > NA_MAX_ITEMS)
    return set_error(nullptr, TC_ERR_UNSUPPORTED,
                     "tc_count_dag_noalloc: %lld edges exceed the limit of %lld edges of its %u-byte static scratch",
                     (long long)m, (long long)(NA_MAX_ITEMS * NA_ITEM), (unsigned)TC_NOALLOC_SCRATCH_BYTES);
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) {
    (void)cudaGetLastError();
    return set_error(nullptr, TC_ERR_NO_DEVICE, "no CUDA device");
  }
  // cudaSetDevice also makes the device's primary context current (the
  // context the runtime launches into), which the set-up below relies on.
  if (cudaSetDevice(device) != cudaSuccess) {
    (void)cudaGetLastError();
    return set_error(nullptr, TC_ERR_INVALID_ARG, "cannot make device %d current", device);
  }
  tc_status st = TC_OK;
  void *scratch = nullptr;
  {
    // Set-up, once per device with that device current: the device address of
    // the static array (its host-side name is only a stand-in).  The address
    // belongs to the device's current context; a new context (after
    // cudaDeviceReset) has the array elsewhere, so the set-up runs again.
    std::lock_guard<std::mutex> lk(g_na_mu);
    const unsigned long long ctx_id = current_ctx_id();
    if (!g_na_ptr[device] || g_na_ctx[device] != ctx_id) {
      void *p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) {
        (void)cudaGetLastError();
        g_na_ptr[device] = nullptr;
        st = set_error(nullptr, TC_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
      } else {
        g_na_ptr[device] = p;
        g_na_ctx[device] = ctx_id;
      }
    }
    scratch = g_na_ptr[device];
  }
  if (st == TC_OK) {
    cudaStream_t s = (cudaStream_t)stream;
    const int blocks = (int)std::min<int64_t>(std::max<int64_t>((items + 255) / 256, 1), 4096);
    noalloc_prep_kernel<<<blocks, 256, 0, s>>>(rowptr, n, m, items, (unsigned char *)scratch,
                                               (unsigned long long *)total);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && items > 0) {
      int dev_sms = 0;
      cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, device);
      noalloc_hash_kernel<<<std::max(dev_sms, 1) * 4, NA_THREADS, 0, s>>>(
          rowptr, colidx, n, m, items, (unsigned char *)scratch, (unsigned long long *)total, edge_counts);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) st = set_error(nullptr, TC_ERR_CUDA, "tc_count_dag_noalloc launch: %s", cudaGetErrorString(e));
  }
  if (prev != device) cudaSetDevice(prev);
  return st;
}
