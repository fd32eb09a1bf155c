// gbdx_sched.cu -- longest-duration-first work order for the fused kernels.
//
// The persistent integrator hands out trajectories from a device counter.  When
// the integration intervals differ (per-trajectory t0/t1), handing out the long
// ones first keeps the tail of the launch made of short trajectories, so lanes
// do not idle while a few long solves finish.  The order is a counting sort of
// |t1 - t0| into NB buckets (descending), built by four small kernels in the
// caller's stream and workspace; ties keep no particular order, which does not
// affect results because trajectories are independent.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gbdx_sched.h"

namespace gbdx {

namespace {

constexpr int kNB = kScheduleBuckets;

__device__ __forceinline__ double duration(const double *t0, const double *t1, int64_t i) {
  return fabs(t1[i] - t0[i]);
}

__global__ void sched_max_kernel(const double *t0, const double *t1, int64_t n,
                                 unsigned long long *dmax_key, int *hist) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (blockIdx.x == 0)
    for (int b = threadIdx.x; b < kNB + 1; b += blockDim.x) hist[b] = 0;
  // Non-negative doubles order like their bit patterns.
  unsigned long long k = 0;
  if (i < n) k = (unsigned long long)__double_as_longlong(duration(t0, t1, i));
  for (int off = 16; off > 0; off >>= 1) {
    unsigned long long o = __shfl_down_sync(0xffffffffu, k, off);
    k = o > k ? o : k;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(dmax_key, k);
}

__device__ __forceinline__ int bucket_of(double d, double dmax) {
  if (!(dmax > 0.0)) return 0;
  int b = int(double(kNB) * (d / dmax));
  b = b < 0 ? 0 : (b > kNB - 1 ? kNB - 1 : b);
  return kNB - 1 - b;  // descending durations
}

__global__ void sched_hist_kernel(const double *t0, const double *t1, int64_t n,
                                  const unsigned long long *dmax_key, int *hist) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double dmax = __longlong_as_double((long long)*dmax_key);
  atomicAdd(hist + bucket_of(duration(t0, t1, i), dmax), 1);
}

// Exclusive scan of kNB counts by one block of kNB threads.
__global__ void sched_scan_kernel(int *hist) {
  __shared__ int s[kNB];
  const int t = threadIdx.x;
  s[t] = hist[t];
  __syncthreads();
  for (int off = 1; off < kNB; off <<= 1) {
    int v = t >= off ? s[t - off] : 0;
    __syncthreads();
    s[t] += v;
    __syncthreads();
  }
  hist[t] = t == 0 ? 0 : s[t - 1];
}

__global__ void sched_scatter_kernel(const double *t0, const double *t1, int64_t n,
                                     const unsigned long long *dmax_key, int *offsets,
                                     int32_t *order) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double dmax = __longlong_as_double((long long)*dmax_key);
  const int pos = atomicAdd(offsets + bucket_of(duration(t0, t1, i), dmax), 1);
  order[pos] = int32_t(i);
}

}  // namespace

size_t schedule_workspace_bytes(int64_t n) {
  return align_up(size_t(n) * sizeof(int32_t), 256) + align_up((kNB + 1) * sizeof(int), 256) +
         256;
}

cudaError_t build_longest_first_order(const double *t0, const double *t1, int64_t n,
                                      void *ws, int32_t **order_out, cudaStream_t s) {
  char *p = static_cast<char *>(ws);
  int32_t *order = reinterpret_cast<int32_t *>(p);
  p += align_up(size_t(n) * sizeof(int32_t), 256);
  int *hist = reinterpret_cast<int *>(p);
  p += align_up((kNB + 1) * sizeof(int), 256);
  unsigned long long *dmax = reinterpret_cast<unsigned long long *>(p);
  cudaError_t e = cudaMemsetAsync(dmax, 0, sizeof *dmax, s);
  if (e != cudaSuccess) return e;
  const int threads = 256;
  const unsigned blocks = unsigned((n + threads - 1) / threads);
  sched_max_kernel<<<blocks, threads, 0, s>>>(t0, t1, n, dmax, hist);
  sched_hist_kernel<<<blocks, threads, 0, s>>>(t0, t1, n, dmax, hist);
  sched_scan_kernel<<<1, kNB, 0, s>>>(hist);
  sched_scatter_kernel<<<blocks, threads, 0, s>>>(t0, t1, n, dmax, hist, order);
  *order_out = order;
  return cudaGetLastError();
}

}  // namespace gbdx
