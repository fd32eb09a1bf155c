// gbdx_launch.h -- host-side launch table shared by the ABI and the kernel
// translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gbdx_common.cuh"

namespace gbdx {

struct LaunchCfg {
  int kernel;  // GBDX_KERNEL_PLAIN or GBDX_KERNEL_FUSED
  int block;   // threads per CTA (fused)
  int grid;    // CTAs (fused)
};

using OdeLaunchFn = cudaError_t (*)(const SolveParams &, const LaunchCfg &, cudaStream_t);
using OdeOccFn = cudaError_t (*)(int block, int *ctas_per_sm);

struct OdeEntry {
  OdeLaunchFn launch;
  OdeOccFn occupancy;
};

OdeEntry find_ode_entry_f32(int solver, int field, int dim);
OdeEntry find_ode_entry_f64(int solver, int field, int dim);
// The Ornstein-Uhlenbeck SDE (diagonal diffusion, virtual Brownian tree), FP32.
OdeEntry find_ode_sde_entry_f32(int solver, int dim);
// The Ornstein-Uhlenbeck SDE driven by the space-time Levy area tree (Euler,
// Heun, Dopri5, Tsit5 use its W; ShARK also its H).
OdeEntry find_ode_sde_levy_entry_f32(int solver, int dim);
// The same with the extended outputs (SaveAt(steps), dense, clip, events).
OdeEntry find_ode_sde_entry_f32_xo(int solver, int dim);
OdeEntry find_ode_sde_levy_entry_f32_xo(int solver, int dim);
// The same kernels with SaveAt(steps=n) / SaveAt(dense=True) outputs.
OdeEntry find_ode_entry_f32_xo(int solver, int field, int dim);
OdeEntry find_ode_entry_f64_xo(int solver, int field, int dim);
// Fill n doubles (or floats) with +inf on stream s.
cudaError_t launch_fill_inf_f64(double *p, int64_t n, cudaStream_t s);
cudaError_t launch_fill_inf_f32(float *p, int64_t n, cudaStream_t s);
// ys = +inf, ts = direction * inf over all [batch, n_save] save slots.
cudaError_t launch_fill_saves_f32(float *ys, double *ts, int64_t batch, int n_save, int dim,
                                  const double *t0, const double *t1, int64_t time_stride,
                                  cudaStream_t s);
cudaError_t launch_fill_saves_f64(double *ys, double *ts, int64_t batch, int n_save, int dim,
                                  const double *t0, const double *t1, int64_t time_stride,
                                  cudaStream_t s);
// DenseInterpolation.evaluate / .derivative over a dense solve's outputs.
struct DenseEvalArgs {
  int64_t batch, Q, q_stride, time_stride;
  int dim, max_steps, left, order;
  const double *t0, *t1, *query, *dense_ts;
  const void *y0, *dense_info;
  const int32_t *dense_n;
  void *out;
};
cudaError_t launch_dense_evaluate(int solver, int dtype, const DenseEvalArgs &A, cudaStream_t s);
using BwdLaunchFn = cudaError_t (*)(const SolveParams &, const BwdParams &, int grid,
                                    cudaStream_t);
using BwdOccFn = cudaError_t (*)(int *ctas_per_sm);
struct BwdEntry {
  BwdLaunchFn launch;
  BwdOccFn occupancy;
};
BwdEntry find_mlp_bwd_entry_d64h128(int solver, bool precise, bool sde);
BwdEntry find_mlp_bwd_entry_d32h64(int solver, bool precise, bool sde);
// grad[p] = compensated sum over CTAs of (psum - pcomp)[cta][p]
cudaError_t launch_reduce_partials(const float *psum, const float *pcomp, int n_cta,
                                   int n_params, float *out, cudaStream_t s);
// BacksolveAdjoint backward (MLP fields).
struct BsParams;
using BsLaunchFn = cudaError_t (*)(const SolveParams &, const BsParams &, int grid,
                                   cudaStream_t);
struct BsEntry {
  BsLaunchFn launch;
  BwdOccFn occupancy;
  int rows;    // trajectories per CTA
  int stages;  // RK stages (stage records per row)
  int rec;     // floats per stage record
  int gfrag;   // W0/W2 read as global B fragments
};
BsEntry find_backsolve_entry_d64h256(int solver, bool precise);
BsEntry find_backsolve_entry_d64h128(int solver, bool precise);
BsEntry find_backsolve_entry_d32h64(int solver, bool precise);
// The plain (one trajectory per thread) backsolve: a_theta and the stage
// accumulators as [n_params][batch] columns in the workspace.
BsEntry find_plain_backsolve_entry(int solver, int D, int H);
// BF16 mma B fragments of B[k][n] = trans ? W[n][k] : W[k][n] (K x N).
cudaError_t launch_frag_prep(const float *W, int ldw, int K, int N, int trans, uint2 *out,
                             cudaStream_t s);
// The same for partials whose weight blocks are in mma-fragment order (MLP
// D -> H -> H -> D, then with `diffusion` the neural SDE's D x D diffusion),
// written to grad in the flat order.
cudaError_t launch_reduce_partials_frag(const float *psum, const float *pcomp, int n_cta, int D,
                                        int H, int diffusion, float *out, cudaStream_t s);
OdeEntry find_mlp_plain_entry(int solver, int D, int H, bool sde);
// The plain (one trajectory per thread) RecursiveCheckpointAdjoint backward:
// full tape, per-trajectory parameter cotangents dP [n_params][batch].
BwdEntry find_mlp_plain_bwd_entry(int solver, int D, int H, bool sde);
// out[p] = compensated sum over the batch of dP[p][:]
cudaError_t launch_reduce_columns(const float *dP, int64_t n_params, int64_t batch, float *out,
                                  cudaStream_t s);
OdeEntry find_mlp_entry_d64h128(int solver, bool precise, bool sde);
// The MLP forward on tcgen05 (128 trajectories per CTA, one per thread).
OdeEntry find_mlp_tc_entry(int solver, int D, int H, bool sde);
OdeEntry find_mlp_entry_d64h256(int solver, bool precise, bool sde);
OdeEntry find_mlp_entry_d32h64(int solver, bool precise, bool sde);
// the extended-output forms (SaveAt(steps / dense), clip controller, events)
OdeEntry find_mlp_xo_entry_d64h128(int solver, bool precise, bool sde);
OdeEntry find_mlp_xo_entry_d64h256(int solver, bool precise, bool sde);
OdeEntry find_mlp_xo_entry_d32h64(int solver, bool precise, bool sde);
// Gradients of the analytic-field solves (y0 and args): the forward with the
// full tape, the RecursiveCheckpointAdjoint and BacksolveAdjoint backwards.
struct AdjParams;
using AdjLaunchFn = cudaError_t (*)(const SolveParams &, const AdjParams &, cudaStream_t);
struct AdjEntry {
  OdeEntry fwd{nullptr, nullptr};  // forward recording the tape
  AdjLaunchFn rc_bwd = nullptr;    // RecursiveCheckpointAdjoint backward
  AdjLaunchFn bs_bwd = nullptr;    // BacksolveAdjoint backward (ODEs)
  int n_args = 0;
};
AdjEntry find_ode_adj_entry_f32(int solver, int field, int dim, bool sde);
AdjEntry find_ode_adj_entry_f64(int solver, int field, int dim);
// out[p] = compensated sum over the batch of rows[b][p] ([batch, n_args]).
cudaError_t launch_reduce_arg_rows_f32(const void *rows, int64_t batch, int n_args, void *out,
                                       cudaStream_t s);
cudaError_t launch_reduce_arg_rows_f64(const void *rows, int64_t batch, int n_args, void *out,
                                       cudaStream_t s);

}  // namespace gbdx
