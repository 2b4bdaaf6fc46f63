// Restatement of the reference project's single-GPU triangle-counting kernel
// for sm_103a — a BASELINE for parity and speed comparison, not engine code.
//
// Follows bs_warp_vertex.cuh:2-35 (one warp per vertex, grid-stride; serial
// loop over v in N+(u); per-lane AccType partials; __syncthreads tree
// reduction over BLOCK_SIZE values; one atomicAdd per block) with the
// intersection of GraphGPU::warp_intersect (successful_push_pull/graph_gpu.h:
// 228-252): the shorter list is the lookup list, each lane binary-searches
// keys lane, lane+32, ... in the longer list.  Launch shape of
// multigpu.cu:203-206: BLOCK_SIZE 256, min(65536, ceil(n / WARPS_PER_BLOCK))
// blocks.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

constexpr int BLOCK_SIZE = 256;
constexpr int WARP_SIZE = 32;
constexpr int WARPS_PER_BLOCK = BLOCK_SIZE / WARP_SIZE;

__device__ __forceinline__ bool binary_search(const int32_t *list, int32_t key, int64_t size) {
  int64_t l = 0, r = size - 1;
  while (r >= l) {
    const int64_t mid = l + (r - l) / 2;
    const int32_t value = list[mid];
    if (value == key) return true;
    if (value < key) l = mid + 1; else r = mid - 1;
  }
  return false;
}

__device__ __forceinline__ uint64_t intersect_num(const int32_t *a, int64_t na, const int32_t *b, int64_t nb) {
  const int lane = threadIdx.x & (WARP_SIZE - 1);
  if (na == 0 || nb == 0) return 0;
  const int32_t *lookup = a, *search = b;
  int64_t lookup_size = na, search_size = nb;
  if (na > nb) {
    lookup = b; search = a;
    lookup_size = nb; search_size = na;
  }
  uint64_t count = 0;
  for (int64_t i = lane; i < lookup_size; i += WARP_SIZE)
    if (binary_search(search, lookup[i], search_size)) count += 1;
  return count;
}

__global__ void warp_vertex(int64_t end, const int64_t *rowptr, const int32_t *col, unsigned long long *total) {
  __shared__ unsigned long long partial_sum[BLOCK_SIZE];
  const int64_t global_warp_idx = ((int64_t)blockDim.x * blockIdx.x + threadIdx.x) / WARP_SIZE;
  const int64_t total_warp_num = (int64_t)gridDim.x * blockDim.x / WARP_SIZE;
  unsigned long long cnt = 0;
  for (int64_t u = global_warp_idx; u < end; u += total_warp_num) {
    const int32_t *u_vector = col + rowptr[u];
    const int64_t u_size = rowptr[u + 1] - rowptr[u];
    for (int64_t k = 0; k < u_size; ++k) {
      const int32_t v = u_vector[k];
      cnt += intersect_num(u_vector, u_size, col + rowptr[v], rowptr[v + 1] - rowptr[v]);
    }
  }
  partial_sum[threadIdx.x] = cnt;
  for (int stride = blockDim.x / 2; stride > 0; stride /= 2) {
    __syncthreads();
    if (threadIdx.x < stride) partial_sum[threadIdx.x] += partial_sum[threadIdx.x + stride];
  }
  if (threadIdx.x == 0) atomicAdd(total, partial_sum[0]);
}

}  // namespace

extern "C" {

// Counts the triangles of an oriented graph already on the device.  Returns
// 0 on success, else the CUDA error code.  *ms receives the kernel time.
int tc_ref_warp_vertex(const int64_t *rowptr, const int32_t *col, int64_t n, uint64_t *total, float *ms) {
  unsigned long long *d_total = nullptr;
  cudaEvent_t a, b;
  cudaError_t e = cudaMalloc(&d_total, sizeof(unsigned long long));
  if (e != cudaSuccess) return (int)e;
  cudaMemset(d_total, 0, sizeof(unsigned long long));
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  int64_t nblocks = (n - 1) / WARPS_PER_BLOCK + 1;
  if (nblocks > 65536) nblocks = 65536;
  if (nblocks < 1) nblocks = 1;
  cudaEventRecord(a);
  warp_vertex<<<(unsigned)nblocks, BLOCK_SIZE>>>(n, rowptr, col, d_total);
  cudaEventRecord(b);
  e = cudaEventSynchronize(b);
  if (e == cudaSuccess) e = cudaGetLastError();
  float t = 0;
  cudaEventElapsedTime(&t, a, b);
  if (ms) *ms = t;
  unsigned long long h = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&h, d_total, sizeof(h), cudaMemcpyDeviceToHost);
  *total = h;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(d_total);
  return (int)e;
}

}  // extern "C"
