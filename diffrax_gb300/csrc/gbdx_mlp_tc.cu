// gbdx_mlp_tc.cu -- MLP-field integrator on the fifth-generation tensor cores
// (tcgen05.mma, accumulators and Runge--Kutta stages in tensor memory).
//
// A CTA of 512 threads integrates a tile of 128 trajectories, four threads per
// trajectory: threads r, r + 128, r + 256, r + 384 own TMEM lane r, i.e. row r
// of every product, and split its columns; each keeps the row's controller
// state and all take the same decisions, so the only exchange is the four
// parts of the error norm.  Per RK stage the MLP field
// D -> H -> H -> D (tanh hidden, identity output) is three tile products
//   acc[128 x N] = A[128 x K] W[N x K]^T
// issued by one thread as tcgen05.mma (kind::f16, BF16 operands in shared
// memory, FP32 accumulator in TMEM): the model's BF16 weights against the
// activation operand held as three BF16 pieces (24 significant bits; one
// product per piece), so the products are exact up to the FP32 accumulation
// and the field is as smooth as an FP32 evaluation -- what the adaptive
// controller needs.  Completion is signalled through an mbarrier
// (bounded waits).  TMEM (512 columns x 128 lanes x 32 bit) holds the stage
// vectors: columns [64 j, 64 j + 64) the stage j = 0..5 of the current step
// (stage 0 as the unscaled FSAL field value f0, stages 1..5 as k_j = h f_j),
// columns [384, 512) the product accumulator, whose first 64 columns after the
// last stage hold the last stage's field (k_6, the next step's f0).
//
// Reference semantics as the other integrators: the loop body
// (diffrax/_integrate.py:365-662), the explicit RK step
// (diffrax/_solver/runge_kutta.py:446-1203, tsit5.py), the PID controller
// (diffrax/_step_size_controller/pid.py:394-567), SaveAt(t0/ts/t1).
#include <cuda_bf16.h>

#include "gbdx_launch.h"
#include "gbdx_mma.cuh"
#include "gbdx_tc.cuh"
#include "gbdx_traj.cuh"

namespace gbdx {
namespace {

constexpr int kD = 64, kH = 128, kM = 128;
constexpr int kSplit = 4;                    // threads per row
constexpr int kThreads = kM * kSplit;
constexpr int kDH = kD / kSplit;             // state components per thread
constexpr int kHH = kH / kSplit;             // hidden columns per thread
constexpr uint32_t kAcc = 384;               // first accumulator column
constexpr uint32_t kWait = 1u << 24;         // polls of a completion barrier

struct TcSmem {
  __nv_bfloat16 w0[kH * kD];                 // layer 0: N = H rows, K = D (BF16 weights)
  __nv_bfloat16 w1[kH * kH];                 // layer 1: N = H, K = H
  __nv_bfloat16 w2[kD * kH];                 // layer 2: N = D, K = H
  // activations as three BF16 pieces (24 significant bits): M rows, K <= H
  __nv_bfloat16 ah[kM * kH], al[kM * kH], al2[kM * kH];
  float b0[kH], b1[kH], b2[kD];
  float pa[kSplit][kM], pb[kSplit][kM];      // per-part error norm parts
  int pn[kSplit][kM];                        // per-part NaN flags of y1
  unsigned long long qidx[kM];               // refill: queue slot of each row
  uint64_t bar;
  uint32_t slot;
  int err;
};

// Per-row state in registers (the row_init / row_control rules of the
// row-tile integrator: FP32 log-domain PID, FP64 times).
struct Row {
  double tprev, tnext, t1, floor1, dtc, tp_old, tn_old, t0s, t1s;
  long long idx;
  float hist1, hist2;
  int active, first, keep, dir, save_index, ts_index, nsteps, nacc, nrej, result, sc, nc;
  int at_dtmin;
};

__device__ __forceinline__ bool running(const Row &R, int max_steps) {
  return R.active && order_key(R.tprev) < order_key(R.t1) && R.result == GBDX_SUCCESSFUL &&
         R.nsteps < max_steps;
}

__device__ void init_row(Row &R, int64_t i, const SolveParams &P) {
  const int64_t ti = i * P.time_stride;
  double a = P.t0[ti], b = P.t1[ti];
  const int dir = (a < b) ? 1 : -1;
  a *= dir;
  b *= dir;
  R.idx = i;
  R.dir = dir;
  R.t1 = b;
  double tn;
  if (P.controller == GBDX_PID) {
    double h = P.dt0 ? P.dt0[ti] * dir : 0.01;
    if (P.has_dtmax) h = fmin(h, P.dtmax);
    if (P.has_dtmin) h = fmax(h, P.dtmin);
    tn = a + h;
    R.hist1 = R.hist2 = 0.f;
  } else {
    const double h = P.dt0[ti] * dir;
    R.sc = 1;
    R.nc = (int)ceil((b - a) / next_up(h));
    R.t0s = a;
    R.t1s = b;
    tn = a + h;
  }
  R.tnext = fmin(tn, b);
  R.dtc = R.tnext - a;
  R.tprev = a;
  R.floor1 = t1_clip_floor(b);
  R.first = 1;
  R.keep = 0;
  R.save_index = 0;
  R.ts_index = 0;
  R.nsteps = R.nacc = R.nrej = 0;
  R.result = GBDX_SUCCESSFUL;
  R.active = 1;
  R.at_dtmin = 0;
  if (P.save_t0) {
    *GBDX_AT(P, P.ts_out, i * P.n_save, 1, P.batch * P.n_save, GBDX_SITE_TS) = a * dir;
    R.save_index = 1;
  }
}

// pid.py:466-567 / constant.py:59-104 / _integrate.py:410-413 for one row,
// given acc = the sum of squared scaled errors over the D components.
__device__ void control_row(Row &R, float acc, const SolveParams &P) {
  const double dt = R.dtc;
  bool keep;
  double nt0, nt1, dtn;
  if (P.controller == GBDX_PID) {
    keep = acc < float(kD);
    const float lg = 0.5f * (log2f(float(kD)) - __log2f(acc));
    float ex = 0.f;
    if (P.c1_f != 0.f) ex += P.c1_f * lg;
    if (P.c2_f != 0.f) ex += P.c2_f * R.hist1;
    if (P.c3_f != 0.f) ex += P.c3_f * R.hist2;
    float factor = P.safety_f * exp2f(ex);
    const float hnew = isinf(lg) ? 0.f : lg;
    if (P.has_dtmin) keep = keep || R.at_dtmin;
    const float fmn = keep ? 1.f : P.factormin_f;
    const float fmx = keep ? P.factormax_f : P.safety_f;
    factor = fminf(fmaxf(factor, fmn), fmx);
    dtn = dt * double(factor);
    if (P.has_dtmax) dtn = fmin(dtn, P.dtmax);
    if (P.has_dtmin) {
      if (!P.force_dtmin && dtn < P.dtmin && R.result == GBDX_SUCCESSFUL)
        R.result = GBDX_DT_MIN_REACHED;
      if (R.at_dtmin && factor == 1.f) dtn = P.dtmin;
      R.at_dtmin = dtn <= P.dtmin;
      dtn = fmax(dtn, P.dtmin);
    }
    nt0 = keep ? R.tnext : R.tprev;
    nt1 = nt0 + dtn;
    if (keep) {
      R.hist2 = R.hist1;
      R.hist1 = hnew;
    }
  } else {
    keep = true;
    const int s2 = R.sc + 1;
    // the reference's rounding: a multiply, then an add (no contraction)
    double tn = __dadd_rn(R.t0s, __dmul_rn(R.t1s - R.t0s, double(s2) / double(R.nc)));
    if (s2 == R.nc) tn = R.t1s;
    R.sc = s2;
    nt0 = R.tnext;
    nt1 = tn;
    dtn = tn - nt0;
  }
  if (order_key(nt1) > order_key(R.floor1)) {
    nt1 = keep ? R.t1 : nt0 + 0.5 * (R.t1 - nt0);
    dtn = nt1 - nt0;
  }
  R.keep = keep;
  R.tp_old = R.tprev;
  R.tn_old = R.tnext;
  if (keep) {
    R.nacc++;
    R.first = 0;
  } else {
    R.nrej++;
  }
  R.nsteps++;
  R.tprev = nt0;
  R.tnext = nt1;
  R.dtc = dtn;
}

// 16 values of this thread's row as three BF16 pieces into the K-major
// operand tiles (two 16-byte runs per piece and half).
__device__ __forceinline__ void put16(TcSmem &sm, int row, int col, int K, const float (&v)[16]) {
  uint32_t p0[8], p1[8], p2[8];
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
    const float2 hf = __bfloat1622float2(h);
    const float r0 = v[2 * j] - hf.x, r1 = v[2 * j + 1] - hf.y;
    const __nv_bfloat162 m = __floats2bfloat162_rn(r0, r1);
    const float2 mf = __bfloat1622float2(m);
    const __nv_bfloat162 l = __floats2bfloat162_rn(r0 - mf.x, r1 - mf.y);
    p0[j] = *reinterpret_cast<const uint32_t *>(&h);
    p1[j] = *reinterpret_cast<const uint32_t *>(&m);
    p2[j] = *reinterpret_cast<const uint32_t *>(&l);
  }
  unsigned char *b0 = reinterpret_cast<unsigned char *>(sm.ah);
  unsigned char *b1 = reinterpret_cast<unsigned char *>(sm.al);
  unsigned char *b2 = reinterpret_cast<unsigned char *>(sm.al2);
#pragma unroll
  for (int half = 0; half < 2; half++) {
    const uint32_t off = tc::kmajor_offset(row, col + 8 * half, K);
    const int q = 4 * half;
    *reinterpret_cast<uint4 *>(b0 + off) = make_uint4(p0[q], p0[q + 1], p0[q + 2], p0[q + 3]);
    *reinterpret_cast<uint4 *>(b1 + off) = make_uint4(p1[q], p1[q + 1], p1[q + 2], p1[q + 3]);
    *reinterpret_cast<uint4 *>(b2 + off) = make_uint4(p2[q], p2[q + 1], p2[q + 2], p2[q + 3]);
  }
}

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16};"
      :: "r"(taddr), "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])),
         "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])),
         "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
         "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])),
         "r"(__float_as_uint(v[11])), "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])),
         "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15]))
      : "memory");
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// Everyone's operand writes are visible to the tensor core, then one thread
// issues acc = (A0 + A1 + A2) W^T as three products per K = 16 slice (one per
// activation piece, all against the BF16 weights) and commits to the
// barrier; all wait (bounded).  Returns false on a timeout.
__device__ __forceinline__ bool layer(TcSmem &sm, uint32_t tmem, const __nv_bfloat16 *w, int K,
                                      int N, uint32_t &phase) {
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc::fence_after_sync();
    const uint32_t idesc = tc::idesc_bf16_f32(kM, N);
    const uint32_t a0 = tc::smem_u32(sm.ah), a1 = tc::smem_u32(sm.al),
                   a2 = tc::smem_u32(sm.al2);
    const uint32_t bw = tc::smem_u32(w);
    const uint32_t sbo = uint32_t(K) * 16u;
    for (int kk = 0; kk < K / 16; kk++) {
      const uint32_t o = 256u * kk;
      const uint64_t db = tc::smem_desc(bw + o, 128u, sbo);
      tc::mma_bf16(tmem + kAcc, tc::smem_desc(a0 + o, 128u, sbo), db, idesc, kk > 0 ? 1u : 0u);
      tc::mma_bf16(tmem + kAcc, tc::smem_desc(a1 + o, 128u, sbo), db, idesc, 1u);
      tc::mma_bf16(tmem + kAcc, tc::smem_desc(a2 + o, 128u, sbo), db, idesc, 1u);
    }
    tc::mma_commit(&sm.bar);
  }
  const bool ok = tc::mbar_wait(&sm.bar, phase, kWait);
  phase ^= 1u;
  tc::fence_after_sync();
  return ok;
}

// Hidden layer epilogue: tanh(acc + b) of this thread's part of its row's
// columns as the next product's operand (K = H).
__device__ __forceinline__ void hidden_epilogue(TcSmem &sm, uint32_t lane_addr, const float *b,
                                                int row, int part) {
#pragma unroll
  for (int c = part * kHH; c < (part + 1) * kHH; c += 16) {
    float v[16];
    tc::tmem_ld16(lane_addr + kAcc + c, v);
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = tanhf(v[j] + b[c + j]);
    put16(sm, row, c, kH, v);
  }
}

// The field at the operand already written (K = D): three layers; the output
// f - b2 is left in accumulator columns [0, D).
__device__ __forceinline__ bool mlp_eval(TcSmem &sm, uint32_t tmem, uint32_t lane_addr, int row,
                                         int part, uint32_t &phase) {
  bool ok = layer(sm, tmem, sm.w0, kD, kH, phase);
  hidden_epilogue(sm, lane_addr, sm.b0, row, part);
  ok &= layer(sm, tmem, sm.w1, kH, kH, phase);
  hidden_epilogue(sm, lane_addr, sm.b1, row, part);
  ok &= layer(sm, tmem, sm.w2, kH, kD, phase);
  return ok;
}

// Stage I's input y + sum_{s<I} a_Is k_s of this thread's part of its row (y first,
// the newest stage last; k_0 = h f0) as the first product's operand.
template <int SOLVER, int I>
__device__ __forceinline__ void stage_input(TcSmem &sm, uint32_t lane_addr, const float (&y)[kDH],
                                            float h, int row, int col0) {
  using TB = Tab<SOLVER>;
#pragma unroll
  for (int c = 0; c < kDH; c += 16) {
    float yi[16], kv[16];
#pragma unroll
    for (int j = 0; j < 16; j++) yi[j] = y[c + j];
#pragma unroll
    for (int s = 0; s < I; s++) {
      if (TB::a(I, s) == 0.0) continue;
      tc::tmem_ld16(lane_addr + 64u * s + col0 + c, kv);
      const float a = float(TB::a(I, s));
#pragma unroll
      for (int j = 0; j < 16; j++) yi[j] = fmaf(a, s == 0 ? kv[j] * h : kv[j], yi[j]);
    }
    put16(sm, row, col0 + c, kD, yi);
  }
}

// kSplit threads integrate each row: thread t handles row t % 128 and the
// part t / 128 of its columns.  Each keeps the row's controller state and all
// take the same decisions (the controller is deterministic in the combined
// error norm, the only value they exchange).
template <int SOLVER>
__global__ void __launch_bounds__(kThreads, 1) mlp_tc_kernel(SolveParams P) {
  using TB = Tab<SOLVER>;
  static_assert(TB::S == 7 && TB::FSAL && TB::SSAL, "seven-stage FSAL/SSAL tableau");
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcSmem &sm = *reinterpret_cast<TcSmem *>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int row = tid & (kM - 1), part = tid >> 7, col0 = part * kDH;
  const float *W = P.mlp;
  constexpr int OW0 = 0, OB0 = OW0 + kH * kD, OW1 = OB0 + kH, OB1 = OW1 + kH * kH,
                OW2 = OB1 + kH, OB2 = OW2 + kD * kH;

  // the BF16 weights in the K-major operand layout, biases
  for (int i = tid; i < kH * kD; i += kThreads) {
    const int n = i / kD, k = i % kD;
    sm.w0[tc::kmajor_offset(n, k, kD) / 2] = __float2bfloat16_rn(W[OW0 + i]);
  }
  for (int i = tid; i < kH * kH; i += kThreads) {
    const int n = i / kH, k = i % kH;
    sm.w1[tc::kmajor_offset(n, k, kH) / 2] = __float2bfloat16_rn(W[OW1 + i]);
  }
  for (int i = tid; i < kD * kH; i += kThreads) {
    const int n = i / kH, k = i % kH;
    sm.w2[tc::kmajor_offset(n, k, kH) / 2] = __float2bfloat16_rn(W[OW2 + i]);
  }
  for (int i = tid; i < kH; i += kThreads) {
    sm.b0[i] = W[OB0 + i];
    sm.b1[i] = W[OB1 + i];
  }
  for (int i = tid; i < kD; i += kThreads) sm.b2[i] = W[OB2 + i];
  if (warp == 0) tc::tmem_alloc(&sm.slot, 512);
  if (tid == 0) {
    tc::mbar_init(&sm.bar, 1);
    sm.err = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = sm.slot;
  // this thread's TMEM lane: warps w and w + 4 share lanes 32 (w % 4) ...
  const uint32_t lane_addr = tmem + (uint32_t((warp & 3) * 32) << 16);
  uint32_t phase = 0;

  Row R;
  float y[kDH];
  R.active = 0;
  R.idx = 0;
  // Take the next trajectory from the queue for rows that need one (`want`):
  // the row's first thread draws the index, both threads load it.
  auto refill = [&](bool want) {
    if (want && part == 0) sm.qidx[row] = atomicAdd(P.queue, 1ull);
    __syncthreads();
    if (!want) return;
    const unsigned long long q = sm.qidx[row];
    if (q < (unsigned long long)P.batch) {
      init_row(R, P.order ? (int64_t)P.order[q] : (int64_t)q, P);
      const float *y0 = reinterpret_cast<const float *>(P.y0) + R.idx * kD + col0;
#pragma unroll
      for (int n = 0; n < kDH; n++) y[n] = y0[n];
      if (P.save_t0) {
        float *o = GBDX_AT(P, reinterpret_cast<float *>(P.ys_out), R.idx * P.n_save * kD + col0,
                           kDH, P.batch * P.n_save * kD, GBDX_SITE_YS);
#pragma unroll
        for (int n = 0; n < kDH; n++) o[n] = y[n];
      }
    } else {
      R.active = 0;
#pragma unroll
      for (int n = 0; n < kDH; n++) y[n] = 0.f;
    }
  };
  refill(true);

  while (true) {
    const bool live = running(R, P.max_steps);
    const float h = live ? float(R.dir > 0 ? R.dtc : -R.dtc) : 0.f;
    // stage 0: a fresh evaluation when some row starts (FSAL otherwise;
    // runge_kutta.py:684-700).  Re-evaluating at y reproduces the FSAL value
    // of the other rows bit for bit.
    if (__syncthreads_or(live && R.first)) {
#pragma unroll
      for (int c = 0; c < kDH; c += 16) {
        float v[16];
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] = y[c + j];
        put16(sm, row, col0 + c, kD, v);
      }
      if (!mlp_eval(sm, tmem, lane_addr, row, part, phase)) sm.err = 1;
#pragma unroll
      for (int c = col0; c < col0 + kDH; c += 16) {
        float v[16];
        tc::tmem_ld16(lane_addr + kAcc + c, v);
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] += sm.b2[c + j];
        tmem_st16(lane_addr + c, v);  // slot 0: f0
      }
    }
    // stages 1..6
#pragma unroll 1
    for (int i = 1; i < 7; i++) {
      switch (i) {
        case 1: stage_input<SOLVER, 1>(sm, lane_addr, y, h, row, col0); break;
        case 2: stage_input<SOLVER, 2>(sm, lane_addr, y, h, row, col0); break;
        case 3: stage_input<SOLVER, 3>(sm, lane_addr, y, h, row, col0); break;
        case 4: stage_input<SOLVER, 4>(sm, lane_addr, y, h, row, col0); break;
        case 5: stage_input<SOLVER, 5>(sm, lane_addr, y, h, row, col0); break;
        default: stage_input<SOLVER, 6>(sm, lane_addr, y, h, row, col0); break;
      }
      if (!mlp_eval(sm, tmem, lane_addr, row, part, phase)) sm.err = 1;
      if (i < 6) {
#pragma unroll
        for (int c = col0; c < col0 + kDH; c += 16) {
          float v[16];
          tc::tmem_ld16(lane_addr + kAcc + c, v);
#pragma unroll
          for (int j = 0; j < 16; j++) v[j] = (v[j] + sm.b2[c + j]) * h;
          tmem_st16(lane_addr + 64u * i + c, v);  // k_i
        }
      }
    }
    // y1 (SSAL: the last stage's input), error estimate and this thread's part of
    // the scaled error norm, both against max(|y0|, |y1|) and (for a row whose
    // y1 has a NaN, pid.py:466-492) against |y0|
    float pa = 0.f, pb = 0.f;
    bool nanf = false;
#pragma unroll
    for (int c = 0; c < kDH; c += 16) {
      float y1[16], er[16], kv[16];
#pragma unroll
      for (int j = 0; j < 16; j++) {
        y1[j] = y[c + j];
        er[j] = 0.f;
      }
#pragma unroll
      for (int s = 0; s < 7; s++) {
        if (s < 6) {
          tc::tmem_ld16(lane_addr + 64u * s + col0 + c, kv);
        } else {
          tc::tmem_ld16(lane_addr + kAcc + col0 + c, kv);
        }
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const float k =
              s == 0 ? kv[j] * h : s == 6 ? (kv[j] + sm.b2[col0 + c + j]) * h : kv[j];
          if (s < 6) y1[j] = fmaf(float(TB::a(6, s)), k, y1[j]);
          if (TB::e(s) != 0.0) er[j] = fmaf(float(TB::e(s)), k, er[j]);
        }
      }
#pragma unroll
      for (int j = 0; j < 16; j++) {
        nanf |= isnan(y1[j]);
        const float e = isnan(er[j]) ? INFINITY : er[j];
        const float a0 = fabsf(y[c + j]);
        const float sa = __fdividef(e, fmaf(fmaxf(a0, fabsf(y1[j])), P.rtol_f, P.atol_f));
        const float sb = __fdividef(e, fmaf(a0, P.rtol_f, P.atol_f));
        pa = fmaf(sa, sa, pa);
        pb = fmaf(sb, sb, pb);
      }
    }
    sm.pa[part][row] = pa;
    sm.pb[part][row] = pb;
    sm.pn[part][row] = nanf ? 1 : 0;
    __syncthreads();
    bool rownan = false;
    float acc_a = 0.f, acc_b = 0.f;
#pragma unroll
    for (int q = 0; q < kSplit; q++) {  // the same order in every thread of the row
      rownan |= sm.pn[q][row] != 0;
      acc_a += sm.pa[q][row];
      acc_b += sm.pb[q][row];
    }
    const float acc = rownan ? acc_b : acc_a;
    if (live) control_row(R, acc, P);
    const bool kept = live && R.keep;
    // SaveAt(ts) inside the step just taken (_integrate.py:456-487)
    while (true) {
      bool pend = false;
      double tsv = 0.0;
      float th = 0.f;
      if (kept && R.ts_index < P.n_ts) {
        tsv = __ldg(P.save_ts + R.ts_index);
        const double tsd = R.dir * tsv;
        if (order_key(tsd) <= order_key(R.tn_old)) {
          pend = true;
          const double tp = R.tp_old, tn = R.tn_old;
          th = float(tp == tn ? 0.0 : (tsd - tp) / (tn - tp));
        }
      }
      if (!__any_sync(0xffffffffu, pend)) break;
      float *o = GBDX_AT(P, reinterpret_cast<float *>(P.ys_out),
                         (R.idx * P.n_save + (pend ? R.save_index : 0)) * kD + col0, kDH,
                         P.batch * P.n_save * kD, GBDX_SITE_YS);
#pragma unroll
      for (int c = 0; c < kDH; c += 16) {
        // Tsit5: y0 + sum_s w_s(theta) k_s (tsit5.py:103-156); Dopri5: the
        // quartic through y0, y1, the midpoint y0 + sum_s cmid_s k_s and the
        // end slopes k_0, k_6 (dopri5.py:36-47, _local_interpolation.py:95-139)
        float v[16], y1[16], kv[16], fa[16];
#pragma unroll
        for (int j = 0; j < 16; j++) {
          v[j] = 0.f;
          y1[j] = y[c + j];
        }
#pragma unroll
        for (int s = 0; s < 7; s++) {
          if (s < 6) tc::tmem_ld16(lane_addr + 64u * s + col0 + c, kv);
          else tc::tmem_ld16(lane_addr + kAcc + col0 + c, kv);
#pragma unroll
          for (int j = 0; j < 16; j++) {
            const float k =
                s == 0 ? kv[j] * h : s == 6 ? (kv[j] + sm.b2[col0 + c + j]) * h : kv[j];
            if constexpr (SOLVER == GBDX_DOPRI5) {
              v[j] = fmaf(float(Tab<GBDX_DOPRI5>::cmid(s)), k, v[j]);
              if (s < 6) y1[j] = fmaf(float(TB::a(6, s)), k, y1[j]);
              if (s == 0) fa[j] = k;
              if (s == 6) {
                const float y0 = y[c + j], ym = y0 + v[j], fb = k;
                const float a = 2.f * (fb - fa[j]) - 8.f * (y1[j] + y0) + 16.f * ym;
                const float b = 5.f * fa[j] - 3.f * fb + 18.f * y0 + 14.f * y1[j] - 32.f * ym;
                const float cc = fb - 4.f * fa[j] - 11.f * y0 - 5.f * y1[j] + 16.f * ym;
                v[j] = (((a * th + b) * th + cc) * th + fa[j]) * th + y0;  // the value
              }
            } else {
              v[j] = fmaf(tsit5_w<float>(s, th), k, v[j]);
            }
          }
        }
        if (pend) {
#pragma unroll
          for (int j = 0; j < 16; j++) o[c + j] = SOLVER == GBDX_DOPRI5 ? v[j] : y[c + j] + v[j];
        }
      }
      if (pend) {
        if (part == 0)
          *GBDX_AT(P, P.ts_out, R.idx * P.n_save + R.save_index, 1, P.batch * P.n_save,
                   GBDX_SITE_TS) = tsv;
        R.ts_index++;
        R.save_index++;
      }
    }
    // accept: y = y1, f0 = the last stage's field (FSAL); a rejected row
    // keeps both
#pragma unroll
    for (int c = 0; c < kDH; c += 16) {
      float y1[16], kv[16];
#pragma unroll
      for (int j = 0; j < 16; j++) y1[j] = y[c + j];
#pragma unroll
      for (int s = 0; s < 6; s++) {
        tc::tmem_ld16(lane_addr + 64u * s + col0 + c, kv);
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const float k = s == 0 ? kv[j] * h : kv[j];
          y1[j] = fmaf(float(TB::a(6, s)), k, y1[j]);
        }
      }
      float f0[16];
      tc::tmem_ld16(lane_addr + col0 + c, f0);
      tc::tmem_ld16(lane_addr + kAcc + col0 + c, kv);
#pragma unroll
      for (int j = 0; j < 16; j++) {
        if (kept) {
          y[c + j] = y1[j];
          f0[j] = kv[j] + sm.b2[col0 + c + j];
        }
      }
      tmem_st16(lane_addr + col0 + c, f0);
    }
    // finished rows: t1 save, unused slots, results; then refill
    const bool fin = R.active && !running(R, P.max_steps);
    if (fin) {
      const int64_t i = R.idx;
      const int dir = R.dir;
      const double t0 = P.t0[i * P.time_stride] * dir;
      float *o = reinterpret_cast<float *>(P.ys_out);
      const int64_t yb = i * P.n_save * kD + col0, ye = P.batch * P.n_save * kD;
      const int64_t te = P.batch * P.n_save;
      int si = R.save_index;
      if (t0 == R.t1) {
        for (int m = 0; m < P.n_ts; m++, si++) {
          if (part == 0) *GBDX_AT(P, P.ts_out, i * P.n_save + si, 1, te, GBDX_SITE_TS) = t0 * dir;
          float *r = GBDX_AT(P, o, yb + si * kD, kDH, ye, GBDX_SITE_YS);
          for (int n = 0; n < kDH; n++) r[n] = y[n];
        }
      }
      if (P.save_t1) {
        if (part == 0)
          *GBDX_AT(P, P.ts_out, i * P.n_save + si, 1, te, GBDX_SITE_TS) = R.tprev * dir;
        float *r = GBDX_AT(P, o, yb + si * kD, kDH, ye, GBDX_SITE_YS);
        for (int n = 0; n < kDH; n++) r[n] = y[n];
        si++;
      }
      for (int m = si; m < P.n_save; m++) {
        if (part == 0)
          *GBDX_AT(P, P.ts_out, i * P.n_save + m, 1, te, GBDX_SITE_TS) =
              dir > 0 ? INFINITY : -INFINITY;
        float *r = GBDX_AT(P, o, yb + m * kD, kDH, ye, GBDX_SITE_YS);
        for (int n = 0; n < kDH; n++) r[n] = INFINITY;
      }
      if (part == 0) {
        int res = R.result;
        if (sm.err) res = GBDX_INTERNAL_ERROR;
        if (res == GBDX_SUCCESSFUL && order_key(R.tprev) < order_key(R.t1))
          res = GBDX_MAX_STEPS_REACHED;
        P.result_out[i] = res;
        P.stats_out[i * 3 + 0] = R.nsteps;
        P.stats_out[i * 3 + 1] = R.nacc;
        P.stats_out[i * 3 + 2] = R.nrej;
      }
      R.active = 0;
    }
    const bool err = sm.err != 0;
    refill(fin && !err);
    if (err && R.active) {
      // a product did not complete: end every row with an internal error
      if (part == 0) P.result_out[R.idx] = GBDX_INTERNAL_ERROR;
      R.active = 0;
    }
    if (!__syncthreads_or(R.active)) break;
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

template <int SOLVER>
cudaError_t launch_tc(const SolveParams &P, const LaunchCfg &cfg, cudaStream_t s) {
  auto k = mlp_tc_kernel<SOLVER>;
  cudaError_t e =
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(TcSmem)));
  if (e != cudaSuccess) return e;
  if (P.batch <= 0) return cudaSuccess;
  k<<<cfg.grid, kThreads, sizeof(TcSmem), s>>>(P);
  return cudaGetLastError();
}

template <int SOLVER>
cudaError_t occupancy_tc(int, int *ctas) {
  auto k = mlp_tc_kernel<SOLVER>;
  cudaError_t e =
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(TcSmem)));
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, k, kThreads, sizeof(TcSmem));
  // one CTA per SM: it holds all 512 TMEM columns
  if (e == cudaSuccess && *ctas > 1) *ctas = 1;
  return e;
}

}  // namespace

OdeEntry find_mlp_tc_entry(int solver, int D, int H, bool sde) {
  if (sde || D != kD || H != kH) return OdeEntry{nullptr, nullptr};
  if (solver == GBDX_TSIT5) return OdeEntry{&launch_tc<GBDX_TSIT5>, &occupancy_tc<GBDX_TSIT5>};
  if (solver == GBDX_DOPRI5) return OdeEntry{&launch_tc<GBDX_DOPRI5>, &occupancy_tc<GBDX_DOPRI5>};
  return OdeEntry{nullptr, nullptr};
}

}  // namespace gbdx
