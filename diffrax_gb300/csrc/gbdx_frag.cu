// gbdx_frag.cu -- BF16 B-operand fragments of a fixed FP32 matrix, arranged
// for mma.m16n8k16 as [n8 tile][k16 tile][lane] (one 8-byte load per lane).
#include "gbdx_launch.h"
#include "gbdx_mma.cuh"

namespace gbdx {

namespace {
// Tile (kt, nt), lane (g = lane / 4, c = lane % 4): {B[2c][g], B[2c+1][g]} and
// {B[2c+8][g], B[2c+9][g]} relative to the tile origin, lower k in the low
// half, with B[k][n] = W[n][k] (trans) or W[k][n].
__global__ void frag_prep_kernel(const float *W, int ldw, int K, int N, int trans, uint2 *out) {
  const int KT = K / 16;
  const int total = (N / 8) * KT * 32;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const int lane = idx & 31, kt = (idx >> 5) % KT, nt = (idx >> 5) / KT;
  const int n = nt * 8 + (lane >> 2), k = kt * 16 + 2 * (lane & 3);
  auto B = [&](int kk) { return trans ? W[size_t(n) * ldw + kk] : W[size_t(kk) * ldw + n]; };
  out[idx] = make_uint2(pack_bf16x2(B(k), B(k + 1)), pack_bf16x2(B(k + 8), B(k + 9)));
}
}  // namespace

cudaError_t launch_frag_prep(const float *W, int ldw, int K, int N, int trans, uint2 *out,
                             cudaStream_t s) {
  const int total = (N / 8) * (K / 16) * 32;
  frag_prep_kernel<<<(total + 255) / 256, 256, 0, s>>>(W, ldw, K, N, trans, out);
  return cudaGetLastError();
}

}  // namespace gbdx
