// gbdx_tc.cu -- a self-test of the fifth-generation tensor-core path on the
// running GPU: one CTA computes D = A B^T (A, B: 128 x 64, BF16 operands in
// shared memory, FP32 accumulator in tensor memory) with tcgen05.mma and reads
// D back with tcgen05.ld.
#include <cuda_bf16.h>

#include "../../include/gbdx.h"
#include "gbdx_tc.cuh"

namespace gbdx {
int set_last_error(int code, const char *msg);

namespace {

constexpr int kM = 128, kN = 128, kK = 64;
constexpr uint32_t kWaitLimit = 1u << 22;  // polls of the completion barrier

__global__ void __launch_bounds__(128) tc_selftest_kernel(const float *A, const float *B,
                                                          float *D, int32_t *status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char *sa = smem;                    // A: 128 x 64 BF16, 16 KB
  unsigned char *sb = smem + kM * kK * 2;      // B: 128 x 64 BF16, 16 KB
  uint64_t *bar = reinterpret_cast<uint64_t *>(sb + kN * kK * 2);
  uint32_t *slot = reinterpret_cast<uint32_t *>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5;

  for (int i = tid; i < kM * kK; i += blockDim.x) {
    const int r = i / kK, k = i % kK;
    *reinterpret_cast<__nv_bfloat16 *>(sa + tc::kmajor_offset(r, k, kK)) =
        __float2bfloat16_rn(A[i]);
    *reinterpret_cast<__nv_bfloat16 *>(sb + tc::kmajor_offset(r, k, kK)) =
        __float2bfloat16_rn(B[i]);
  }
  if (warp == 0) tc::tmem_alloc(slot, kN);
  if (tid == 0) tc::mbar_init(bar, 1);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *slot;
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_bf16_f32(kM, kN);
    const uint32_t a0 = tc::smem_u32(sa), b0 = tc::smem_u32(sb);
    for (int kk = 0; kk < kK / 16; kk++) {
      const uint64_t da = tc::smem_desc(a0 + 256u * kk, 128u, kK * 16u);
      const uint64_t db = tc::smem_desc(b0 + 256u * kk, 128u, kK * 16u);
      tc::mma_bf16(tmem, da, db, idesc, kk > 0 ? 1u : 0u);
    }
    tc::mma_commit(bar);
  }
  const bool ok = tc::mbar_wait(bar, 0, kWaitLimit);
  tc::fence_after_sync();
  if (!ok) {
    if (tid == 0) *status = 1;  // the products did not complete in time
  } else {
    const int row = tid;  // warp w reads TMEM lanes 32 w .. 32 w + 31
    for (int c = 0; c < kN; c += 16) {
      float v[16];
      tc::tmem_ld16(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c), v);
#pragma unroll
      for (int j = 0; j < 16; j++) D[row * kN + c + j] = v[j];
    }
    if (tid == 0) *status = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kN);
}

}  // namespace
}  // namespace gbdx

extern "C" int gbdx_selftest_tcgen05(const float *A, const float *B, float *D, int32_t *status,
                                     void *stream) {
  if (!A || !B || !D || !status)
    return gbdx::set_last_error(GBDX_ERR_INVALID, "null pointer argument");
  const size_t smem = size_t(128 * 64 * 2) * 2 + 64;
  cudaError_t e = cudaFuncSetAttribute(gbdx::tc_selftest_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e == cudaSuccess) {
    gbdx::tc_selftest_kernel<<<1, 128, smem, reinterpret_cast<cudaStream_t>(stream)>>>(
        A, B, D, status);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return gbdx::set_last_error(GBDX_ERR_CUDA, cudaGetErrorString(e));
  return GBDX_OK;
}
