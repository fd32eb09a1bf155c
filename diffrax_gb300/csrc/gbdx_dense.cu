// gbdx_dense.cu -- SaveAt(dense=True) support: the +inf fill of the dense
// buffers before a solve, and DenseInterpolation.evaluate / .derivative
// (diffrax/_global_interpolation.py:315-393) over the recorded steps.
//
// A dense solve records per trajectory the loop's step times
// dense_ts [max_steps + 1] (time runs forward: t * sign(t1 - t0)) and per
// accepted step (y0, y1, k_0 .. k_{S-1}) (diffrax/_integrate.py:529-540).  One
// thread evaluates one (trajectory, query): a binary search of the query in the
// trajectory's step times (the reference's searchsorted, _interpret_t), then the
// solver's local interpolant of that step (tsit5.py:103-156,
// _local_interpolation.py:29-139) or its time derivative.
#include "gbdx_launch.h"
#include "gbdx_traj.cuh"

namespace gbdx {

namespace {

template <class T>
__global__ void fill_inf_kernel(T *p, int64_t n) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    p[i] = T(INFINITY);
}

template <class T>
cudaError_t fill_inf(T *p, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  int64_t blocks = (n + 255) / 256;
  const int64_t cap = int64_t(sms) * 8;  // grid-stride over 8 CTAs of 256 per SM
  if (blocks > cap) blocks = cap;
  fill_inf_kernel<T><<<(unsigned)blocks, 256, 0, s>>>(p, n);
  return cudaGetLastError();
}

// The save buffers of a solve with many save slots (SaveAt(steps=n)): every
// slot starts as the reference's unused save, ys = +inf and ts = direction *
// inf (_integrate.py:1273-1293); the solve overwrites the slots it saves.  One
// coalesced pass here replaces the per-trajectory fill loop at the end of each
// trajectory, which runs on one lane of a warp at a time.
template <class T>
__global__ void fill_saves_kernel(T *ys, double *ts, int64_t batch, int n_save, int dim,
                                  const double *t0, const double *t1, int64_t time_stride) {
  const int64_t n = batch * n_save;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  const int64_t first = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  for (int64_t i = first; i < n; i += stride) {
    const int64_t ti = (i / n_save) * time_stride;
    ts[i] = __ldg(t0 + ti) < __ldg(t1 + ti) ? INFINITY : -INFINITY;
  }
  // ys as one flat array: consecutive threads write consecutive elements
  const int64_t ny = n * dim;
  for (int64_t i = first; i < ny; i += stride) ys[i] = T(INFINITY);
}

template <class T>
cudaError_t fill_saves(T *ys, double *ts, int64_t batch, int n_save, int dim, const double *t0,
                       const double *t1, int64_t time_stride, cudaStream_t s) {
  const int64_t n = batch * int64_t(n_save);
  if (n <= 0) return cudaSuccess;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  int64_t blocks = (n + 255) / 256;
  const int64_t cap = int64_t(sms) * 8;
  if (blocks > cap) blocks = cap;
  fill_saves_kernel<T><<<(unsigned)blocks, 256, 0, s>>>(ys, ts, batch, n_save, dim, t0, t1,
                                                        time_stride);
  return cudaGetLastError();
}

// Value (ORDER 0) or d/dtheta (ORDER 1) of the local interpolant of one step,
// component n of the record r = (y0, y1, k_0 .. k_{S-1}).
template <int SOLVER, class T>
__device__ __forceinline__ T local_interp(const T *r, int D, int n, T th, int order) {
  constexpr int S = Tab<SOLVER>::S;
  const T y0 = r[n], y1 = r[D + n];
  auto k = [&](int j) { return r[(2 + j) * D + n]; };
  if constexpr (SOLVER == GBDX_DOPRI8) {
    T acc = T(0);
#pragma unroll
    for (int j = 0; j < S; j++) acc += (order ? dopri8_dw<T>(j, th) : dopri8_w<T>(j, th)) * k(j);
    return order ? acc : y0 + acc;
  } else if constexpr (SOLVER == GBDX_TSIT5) {
    T acc = T(0);
#pragma unroll
    for (int j = 0; j < 7; j++) acc += (order ? tsit5_dw<T>(j, th) : tsit5_w<T>(j, th)) * k(j);
    return order ? acc : y0 + acc;
  } else if constexpr (SOLVER == GBDX_DOPRI5) {
    // FourthOrderPolynomialInterpolation (_local_interpolation.py:95-139):
    // y(th) = (((a th + b) th + c) th + f0) th + y0
    T cm = T(0);
#pragma unroll
    for (int j = 0; j < S; j++) cm += T(Tab<GBDX_DOPRI5>::cmid(j)) * k(j);
    const T ymid = y0 + cm, fa = k(0), fb = k(S - 1);
    const T a = T(2) * (fb - fa) - T(8) * (y1 + y0) + T(16) * ymid;
    const T b = T(5) * fa - T(3) * fb + T(18) * y0 + T(14) * y1 - T(32) * ymid;
    const T c = fb - T(4) * fa - T(11) * y0 - T(5) * y1 + T(16) * ymid;
    if (order) return ((T(4) * a * th + T(3) * b) * th + T(2) * c) * th + fa;
    return (((a * th + b) * th + c) * th + fa) * th + y0;
  } else if constexpr (SOLVER == GBDX_HEUN) {
    // ThirdOrderHermitePolynomialInterpolation.from_k (:50-92)
    const T ka = k(0), kb = k(S - 1);
    const T a = ka + kb + T(2) * y0 - T(2) * y1;
    const T b = T(-2) * ka - kb - T(3) * y0 + T(3) * y1;
    if (order) return (T(3) * a * th + T(2) * b) * th + ka;
    return ((a * th + b) * th + ka) * th + y0;
  } else {
    // LocalLinearInterpolation (:29-47)
    if (order) return y1 - y0;
    return y0 + th * (y1 - y0);
  }
}

template <int SOLVER, class T>
__global__ void __launch_bounds__(256) dense_eval_kernel(DenseEvalArgs A) {
  constexpr int S = Tab<SOLVER>::S;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= A.batch * A.Q) return;
  const int64_t b = i / A.Q, m = i - b * A.Q;
  const int D = A.dim;
  const double a0 = A.t0[b * A.time_stride], a1 = A.t1[b * A.time_stride];
  const int dir = a0 < a1 ? 1 : -1;
  const int64_t L = int64_t(A.max_steps) + 1;
  const double *ts = A.dense_ts + b * L;
  const int size = A.dense_n[b];
  const double t = A.query[b * A.q_stride + m] * dir;
  T *o = static_cast<T *>(A.out) + i * D;
  // A solve with no step evaluates to y0 at t0 (_global_interpolation.py:344-345).
  if (size == 1 && t == a0 * dir) {
    const T *y0 = static_cast<const T *>(A.y0) + b * D;
    for (int n = 0; n < D; n++) o[n] = A.order ? T(0) : y0[n];
    return;
  }
  // NaN outside [ts[0], ts[size - 1]] (_nan_if_out_of_bounds).
  if (size <= 1 || t < ts[0] || t > ts[size - 1]) {
    for (int n = 0; n < D; n++) o[n] = T(NAN);
    return;
  }
  // index = searchsorted(ts, t, side) - 1, clipped to the recorded steps
  // (_interpret_t); entries past size are +inf and never below t.
  int lo = 0, hi = size;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    const double v = ts[mid];
    const bool right = A.left ? (v < t) : (v <= t);
    if (right) lo = mid + 1; else hi = mid;
  }
  int idx = lo - 1;
  if (idx < 0) idx = 0;
  if (idx > size - 2) idx = size - 2;
  const double tp = ts[idx], tn = ts[idx + 1];
  const double span = tn - tp;
  const T th = T(span == 0.0 ? 0.0 : (t - tp) / span);  // linear_rescale (_misc.py:71-82)
  const T *r = static_cast<const T *>(A.dense_info) + (b * (L - 1) + idx) * int64_t((2 + S) * D);
  if (A.order == 0) {
    for (int n = 0; n < D; n++) o[n] = local_interp<SOLVER, T>(r, D, n, th, 0);
  } else {
    // d/dt = dir * (d/dtheta) / span, back in the caller's time direction
    for (int n = 0; n < D; n++) {
      const T v = local_interp<SOLVER, T>(r, D, n, th, 1);
      o[n] = span == 0.0 ? T(0) : T(double(dir) * double(v) / span);
    }
  }
}

template <class T>
cudaError_t dense_eval_t(int solver, const DenseEvalArgs &A, cudaStream_t s) {
  const int64_t n = A.batch * A.Q;
  if (n <= 0) return cudaSuccess;
  const unsigned blocks = unsigned((n + 255) / 256);
  switch (solver) {
    case GBDX_EULER: dense_eval_kernel<GBDX_EULER, T><<<blocks, 256, 0, s>>>(A); break;
    case GBDX_HEUN: dense_eval_kernel<GBDX_HEUN, T><<<blocks, 256, 0, s>>>(A); break;
    case GBDX_DOPRI5: dense_eval_kernel<GBDX_DOPRI5, T><<<blocks, 256, 0, s>>>(A); break;
    case GBDX_TSIT5: dense_eval_kernel<GBDX_TSIT5, T><<<blocks, 256, 0, s>>>(A); break;
    case GBDX_DOPRI8: dense_eval_kernel<GBDX_DOPRI8, T><<<blocks, 256, 0, s>>>(A); break;
    // the additive-noise SRKs interpolate linearly (srk.py:268, 670)
    case GBDX_SHARK: dense_eval_kernel<GBDX_SHARK, T><<<blocks, 256, 0, s>>>(A); break;
    case GBDX_SRA1: dense_eval_kernel<GBDX_SRA1, T><<<blocks, 256, 0, s>>>(A); break;
    case GBDX_SEA: dense_eval_kernel<GBDX_SEA, T><<<blocks, 256, 0, s>>>(A); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_fill_inf_f64(double *p, int64_t n, cudaStream_t s) { return fill_inf(p, n, s); }
cudaError_t launch_fill_inf_f32(float *p, int64_t n, cudaStream_t s) { return fill_inf(p, n, s); }
cudaError_t launch_fill_saves_f32(float *ys, double *ts, int64_t batch, int n_save, int dim,
                                  const double *t0, const double *t1, int64_t time_stride,
                                  cudaStream_t s) {
  return fill_saves(ys, ts, batch, n_save, dim, t0, t1, time_stride, s);
}
cudaError_t launch_fill_saves_f64(double *ys, double *ts, int64_t batch, int n_save, int dim,
                                  const double *t0, const double *t1, int64_t time_stride,
                                  cudaStream_t s) {
  return fill_saves(ys, ts, batch, n_save, dim, t0, t1, time_stride, s);
}

cudaError_t launch_dense_evaluate(int solver, int dtype, const DenseEvalArgs &A, cudaStream_t s) {
  return dtype == GBDX_F32 ? dense_eval_t<float>(solver, A, s) : dense_eval_t<double>(solver, A, s);
}

}  // namespace gbdx
