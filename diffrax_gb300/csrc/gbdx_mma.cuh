// gbdx_mma.cuh -- warp-level BF16 tensor-core tile products for the MLP
// vector fields (mma.sync.m16n8k16, FP32 accumulate) with ldmatrix operand
// loads from padded shared memory.
//
// Fragment layout of one m16n8 accumulator tile held by a warp (g = lane / 4,
// c = lane % 4): c[0], c[1] -> (row g, cols 2c, 2c+1); c[2], c[3] ->
// (row g + 8, cols 2c, 2c+1).
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace gbdx {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// A fragment of a 16x16 bf16 tile from row-major smem (row stride `ld` elements).
__device__ __forceinline__ void ldsm_a(uint32_t (&a)[4], const __nv_bfloat16 *base, int ld,
                                       int lane) {
  const __nv_bfloat16 *p = base + (lane & 15) * ld + (lane >> 4) * 8;
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(a[0]), "=r"(a[1]), "=r"(a[2]), "=r"(a[3])
               : "r"(smem_u32(p)));
}

// B fragments of two adjacent n8 tiles (16 x 16 of W, W row-major [n][k]).
// b[0..1] -> n tile 0, b[2..3] -> n tile 1.
__device__ __forceinline__ void ldsm_b2(uint32_t (&b)[4], const __nv_bfloat16 *base, int ld,
                                        int lane) {
  // lanes 0-7: n 0-7 @ k0; 8-15: n 0-7 @ k0+8; 16-23: n 8-15 @ k0; 24-31: n 8-15 @ k0+8
  const int n = (lane & 7) + ((lane >> 4) << 3);
  const int k = ((lane >> 3) & 1) * 8;
  const __nv_bfloat16 *p = base + n * ld + k;
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(b[0]), "=r"(b[1]), "=r"(b[2]), "=r"(b[3])
               : "r"(smem_u32(p)));
}

// B fragment of one n8 tile.
__device__ __forceinline__ void ldsm_b1(uint32_t (&b)[2], const __nv_bfloat16 *base, int ld,
                                        int lane) {
  const int n = lane & 7;
  const int k = ((lane >> 3) & 1) * 8;
  const __nv_bfloat16 *p = base + n * ld + k;
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(b[0]), "=r"(b[1])
               : "r"(smem_u32(p)));
}

// A fragment of the TRANSPOSE of a row-major smem matrix G [m][o]: the 16x16
// tile with rows o0..o0+15 and columns (k) m0..m0+15 of G^T.
__device__ __forceinline__ void ldsm_at(uint32_t (&a)[4], const __nv_bfloat16 *G, int ld,
                                        int m0, int o0, int lane) {
  const int m = m0 + (lane & 7) + ((lane >> 4) << 3);
  const int o = o0 + ((lane >> 3) & 1) * 8;
  const __nv_bfloat16 *p = G + m * ld + o;
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(a[0]), "=r"(a[1]), "=r"(a[2]), "=r"(a[3])
               : "r"(smem_u32(p)));
}

// B fragments of two adjacent n8 tiles of a K x N operand stored row-major as
// [k][n] in smem (e.g. a weight W [in][out] read as W^T, or activations
// [row][feature] as the K = rows operand): k0..k0+15, n0..n0+15.
__device__ __forceinline__ void ldsm_bt2(uint32_t (&b)[4], const __nv_bfloat16 *S, int ld,
                                         int k0, int n0, int lane) {
  const int k = k0 + (lane & 7) + ((lane >> 3) & 1) * 8;
  const int n = n0 + ((lane >> 4) << 3);
  const __nv_bfloat16 *p = S + k * ld + n;
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(b[0]), "=r"(b[1]), "=r"(b[2]), "=r"(b[3])
               : "r"(smem_u32(p)));
}

// B fragment of one n8 tile of a [k][n] row-major operand.
__device__ __forceinline__ void ldsm_bt1(uint32_t (&b)[2], const __nv_bfloat16 *S, int ld,
                                         int k0, int n0, int lane) {
  const int k = k0 + (lane & 7) + ((lane >> 3) & 1) * 8;
  const __nv_bfloat16 *p = S + k * ld + n0;
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(b[0]), "=r"(b[1])
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&v);
}

// x ~ hi + lo with hi = bf16(x), lo = bf16(x - hi): about 16 significant bits.
__device__ __forceinline__ void split_store(float x, __nv_bfloat16 *hi, __nv_bfloat16 *lo) {
  const __nv_bfloat16 h = __float2bfloat16_rn(x);
  *hi = h;
  if (lo) *lo = __float2bfloat16_rn(x - __bfloat162float(h));
}

// x ~ p0 + p1 + p2, three BF16 pieces (p0 = bf16(x), p1 = bf16(x - p0),
// p2 = bf16(x - p0 - p1)): 24 significant bits, so a product with a BF16
// value is exact up to the FP32 accumulation.  p2 may be null (two pieces).
__device__ __forceinline__ void split_store3(float x, __nv_bfloat16 *p0, __nv_bfloat16 *p1,
                                             __nv_bfloat16 *p2) {
  const __nv_bfloat16 h = __float2bfloat16_rn(x);
  const float r = x - __bfloat162float(h);
  const __nv_bfloat16 m = __float2bfloat16_rn(r);
  *p0 = h;
  *p1 = m;
  if (p2) *p2 = __float2bfloat16_rn(r - __bfloat162float(m));
}

// Two adjacent values as three (or, p2 null, two) BF16x2 pieces.
__device__ __forceinline__ void store_split3x2(float x0, float x1, __nv_bfloat16 *p0,
                                               __nv_bfloat16 *p1, __nv_bfloat16 *p2) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
  const float2 hf = __bfloat1622float2(h);
  const float r0 = x0 - hf.x, r1 = x1 - hf.y;
  const __nv_bfloat162 m = __floats2bfloat162_rn(r0, r1);
  *reinterpret_cast<__nv_bfloat162 *>(p0) = h;
  *reinterpret_cast<__nv_bfloat162 *>(p1) = m;
  if (p2) {
    const float2 mf = __bfloat1622float2(m);
    *reinterpret_cast<__nv_bfloat162 *>(p2) = __floats2bfloat162_rn(r0 - mf.x, r1 - mf.y);
  }
}

// Two adjacent values as hi/lo BF16x2 words.
__device__ __forceinline__ void store_split2(float x0, float x1, __nv_bfloat16 *hi,
                                             __nv_bfloat16 *lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
  const float2 hf = __bfloat1622float2(h);
  const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - hf.x, x1 - hf.y);
  *reinterpret_cast<__nv_bfloat162 *>(hi) = h;
  *reinterpret_cast<__nv_bfloat162 *>(lo) = l;
}

__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// C[16 mt .. +16, 8 nt .. +8*NTW) += A[16 rows, K] * W[8 nt.., K]^T for NTW
// adjacent n8 tiles (NTW even uses x4 B loads).
template <int K, int NTW>
__device__ __forceinline__ void warp_tile_gemm(float (&acc)[NTW][4], const __nv_bfloat16 *A,
                                               int lda, const __nv_bfloat16 *W, int ldw,
                                               int lane) {
#pragma unroll
  for (int kk = 0; kk < K / 16; kk++) {
    uint32_t a[4];
    ldsm_a(a, A + kk * 16, lda, lane);
    if constexpr (NTW % 2 == 0) {
#pragma unroll
      for (int j = 0; j < NTW; j += 2) {
        uint32_t b[4];
        ldsm_b2(b, W + (j * 8) * ldw + kk * 16, ldw, lane);
        mma_bf16(acc[j], a, b[0], b[1]);
        mma_bf16(acc[j + 1], a, b[2], b[3]);
      }
    } else {
#pragma unroll
      for (int j = 0; j < NTW; j++) {
        uint32_t b[2];
        ldsm_b1(b, W + (j * 8) * ldw + kk * 16, ldw, lane);
        mma_bf16(acc[j], a, b[0], b[1]);
      }
    }
  }
}

// acc[j] += A[16 rows at a_row0, K] * B[K, 8 (n0 + 8 j)], with A row-major
// [row][k] and B row-major [k][n] (transposed loads).
template <int K, int NTW>
__device__ __forceinline__ void warp_tile_gemm_bt(float (&acc)[NTW][4], const __nv_bfloat16 *A,
                                                  int lda, const __nv_bfloat16 *B, int ldb,
                                                  int n0, int lane) {
#pragma unroll
  for (int kk = 0; kk < K / 16; kk++) {
    uint32_t a[4];
    ldsm_a(a, A + kk * 16, lda, lane);
    if constexpr (NTW % 2 == 0) {
#pragma unroll
      for (int j = 0; j < NTW; j += 2) {
        uint32_t b[4];
        ldsm_bt2(b, B, ldb, kk * 16, n0 + j * 8, lane);
        mma_bf16(acc[j], a, b[0], b[1]);
        mma_bf16(acc[j + 1], a, b[2], b[3]);
      }
    } else {
#pragma unroll
      for (int j = 0; j < NTW; j++) {
        uint32_t b[2];
        ldsm_bt1(b, B, ldb, kk * 16, n0 + j * 8, lane);
        mma_bf16(acc[j], a, b[0], b[1]);
      }
    }
  }
}

// acc[j] += G^T[16 outputs at o0, M rows] * S[M rows, 8 (n0 + 8 j)]: weight
// gradient tiles (K = the M rows of the tile).
template <int M, int NTW>
__device__ __forceinline__ void warp_tile_gemm_tt(float (&acc)[NTW][4], const __nv_bfloat16 *G,
                                                  int ldg, int o0, const __nv_bfloat16 *S,
                                                  int lds, int n0, int lane) {
#pragma unroll
  for (int kk = 0; kk < M / 16; kk++) {
    uint32_t a[4];
    ldsm_at(a, G, ldg, kk * 16, o0, lane);
    if constexpr (NTW % 2 == 0) {
#pragma unroll
      for (int j = 0; j < NTW; j += 2) {
        uint32_t b[4];
        ldsm_bt2(b, S, lds, kk * 16, n0 + j * 8, lane);
        mma_bf16(acc[j], a, b[0], b[1]);
        mma_bf16(acc[j + 1], a, b[2], b[3]);
      }
    } else {
#pragma unroll
      for (int j = 0; j < NTW; j++) {
        uint32_t b[2];
        ldsm_bt1(b, S, lds, kk * 16, n0 + j * 8, lane);
        mma_bf16(acc[j], a, b[0], b[1]);
      }
    }
  }
}

// acc += (A0 + A1 [+ A2])[16 rows, K] W[8 n tiles, K]^T: an activation held as
// NP BF16 pieces times single-BF16 weights, each W fragment loaded once for
// all pieces.
template <int K, int NTW, int NP>
__device__ __forceinline__ void warp_tile_gemm_p(float (&acc)[NTW][4], const __nv_bfloat16 *A0,
                                                 const __nv_bfloat16 *A1,
                                                 const __nv_bfloat16 *A2, int lda,
                                                 const __nv_bfloat16 *W, int ldw, int lane) {
  static_assert(NP == 2 || NP == 3, "two or three pieces");
#pragma unroll
  for (int kk = 0; kk < K / 16; kk++) {
    uint32_t a[NP][4];
    ldsm_a(a[0], A0 + kk * 16, lda, lane);
    ldsm_a(a[1], A1 + kk * 16, lda, lane);
    if constexpr (NP == 3) ldsm_a(a[NP - 1], A2 + kk * 16, lda, lane);
    if constexpr (NTW % 2 == 0) {
#pragma unroll
      for (int j = 0; j < NTW; j += 2) {
        uint32_t b[4];
        ldsm_b2(b, W + (j * 8) * ldw + kk * 16, ldw, lane);
#pragma unroll
        for (int p = 0; p < NP; p++) {
          mma_bf16(acc[j], a[p], b[0], b[1]);
          mma_bf16(acc[j + 1], a[p], b[2], b[3]);
        }
      }
    } else {
#pragma unroll
      for (int j = 0; j < NTW; j++) {
        uint32_t b[2];
        ldsm_b1(b, W + (j * 8) * ldw + kk * 16, ldw, lane);
#pragma unroll
        for (int p = 0; p < NP; p++) mma_bf16(acc[j], a[p], b[0], b[1]);
      }
    }
  }
}

// acc[j] += (A0 + A1 [+ A2])[16 rows, K] B[K, 8 (nt0 + j)] where the B
// fragments of a fixed BF16 matrix are pre-arranged in global memory as
// [n8 tile][k16 tile][lane] (one 8-byte load per lane, L2-resident).
template <int K, int NTW, int NP>
__device__ __forceinline__ void gemm_gfrag_p(float (&acc)[NTW][4], const __nv_bfloat16 *A0,
                                             const __nv_bfloat16 *A1, const __nv_bfloat16 *A2,
                                             int lda, const uint2 *frag, int nt0, int lane) {
  static_assert(NP == 2 || NP == 3, "two or three pieces");
#pragma unroll 4
  for (int kk = 0; kk < K / 16; kk++) {
    uint32_t a[NP][4];
    ldsm_a(a[0], A0 + kk * 16, lda, lane);
    ldsm_a(a[1], A1 + kk * 16, lda, lane);
    if constexpr (NP == 3) ldsm_a(a[NP - 1], A2 + kk * 16, lda, lane);
#pragma unroll
    for (int j = 0; j < NTW; j++) {
      const uint2 b = __ldg(frag + (size_t((nt0 + j) * (K / 16) + kk) << 5) + lane);
#pragma unroll
      for (int p = 0; p < NP; p++) mma_bf16(acc[j], a[p], b.x, b.y);
    }
  }
}

// acc[j] += (A0 + A1 + A2)[16 rows, K] B[K, 8 (n0 + 8 j)] with B row-major
// [k][n] (transposed loads): a cotangent in three pieces times the weights.
template <int K, int NTW>
__device__ __forceinline__ void warp_tile_gemm_bt3(float (&acc)[NTW][4],
                                                   const __nv_bfloat16 *A0,
                                                   const __nv_bfloat16 *A1,
                                                   const __nv_bfloat16 *A2, int lda,
                                                   const __nv_bfloat16 *B, int ldb, int n0,
                                                   int lane) {
#pragma unroll
  for (int kk = 0; kk < K / 16; kk++) {
    uint32_t a[3][4];
    ldsm_a(a[0], A0 + kk * 16, lda, lane);
    ldsm_a(a[1], A1 + kk * 16, lda, lane);
    ldsm_a(a[2], A2 + kk * 16, lda, lane);
    if constexpr (NTW % 2 == 0) {
#pragma unroll
      for (int j = 0; j < NTW; j += 2) {
        uint32_t b[4];
        ldsm_bt2(b, B, ldb, kk * 16, n0 + j * 8, lane);
#pragma unroll
        for (int p = 0; p < 3; p++) {
          mma_bf16(acc[j], a[p], b[0], b[1]);
          mma_bf16(acc[j + 1], a[p], b[2], b[3]);
        }
      }
    } else {
#pragma unroll
      for (int j = 0; j < NTW; j++) {
        uint32_t b[2];
        ldsm_bt1(b, B, ldb, kk * 16, n0 + j * 8, lane);
#pragma unroll
        for (int p = 0; p < 3; p++) mma_bf16(acc[j], a[p], b[0], b[1]);
      }
    }
  }
}

// acc[j] += (G0 + G1 + G2)^T (S0 + S1 + S2) over M rows (weight-gradient
// tiles) to 24 significant bits: the six piece products whose size is at
// least 2^-18 of the leading one (G0S0, G0S1, G1S0, G0S2, G2S0, G1S1).
template <int M, int NTW>
__device__ __forceinline__ void warp_tile_gemm_tt3(float (&acc)[NTW][4],
                                                   const __nv_bfloat16 *const (&G)[3], int ldg,
                                                   int o0, const __nv_bfloat16 *const (&S)[3],
                                                   int lds, int n0, int lane) {
  constexpr int PAIRS[6][2] = {{0, 0}, {0, 1}, {1, 0}, {0, 2}, {2, 0}, {1, 1}};
#pragma unroll
  for (int kk = 0; kk < M / 16; kk++) {
    uint32_t a[3][4];
#pragma unroll
    for (int p = 0; p < 3; p++) ldsm_at(a[p], G[p], ldg, kk * 16, o0, lane);
    if constexpr (NTW % 2 == 0) {
#pragma unroll
      for (int j = 0; j < NTW; j += 2) {
        uint32_t b[3][4];
#pragma unroll
        for (int p = 0; p < 3; p++) ldsm_bt2(b[p], S[p], lds, kk * 16, n0 + j * 8, lane);
#pragma unroll
        for (int q = 0; q < 6; q++) {
          mma_bf16(acc[j], a[PAIRS[q][0]], b[PAIRS[q][1]][0], b[PAIRS[q][1]][1]);
          mma_bf16(acc[j + 1], a[PAIRS[q][0]], b[PAIRS[q][1]][2], b[PAIRS[q][1]][3]);
        }
      }
    } else {
#pragma unroll
      for (int j = 0; j < NTW; j++) {
        uint32_t b[3][2];
#pragma unroll
        for (int p = 0; p < 3; p++) ldsm_bt1(b[p], S[p], lds, kk * 16, n0 + j * 8, lane);
#pragma unroll
        for (int q = 0; q < 6; q++)
          mma_bf16(acc[j], a[PAIRS[q][0]], b[PAIRS[q][1]][0], b[PAIRS[q][1]][1]);
      }
    }
  }
}

}  // namespace gbdx
