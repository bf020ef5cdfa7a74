// plbm_launch.h — host-visible launch entry points of the device code.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "plbm_params.h"

namespace plbm {

// One timestep of algorithm `alg` (0 nptl, 1 lptl, 2 npol, 3 nsol) for precision `prec` and
// layout `lay`; `t` is the absolute step index (selects the nsol parity kernel).
// porous: the obstacle-select gather of the shifted forms (f32, f16s, bf16s)
cudaError_t launch_nptl(int prec, int lay, const StepParams &p, dim3 grid, dim3 block, cudaStream_t s, bool porous);
cudaError_t launch_lptl(int prec, int lay, const StepParams &p, dim3 grid, dim3 block, cudaStream_t s, bool porous);
// counts[0] = 32-node row segments holding fluid, counts[1] = those mixing interior nodes with and
// without a solid neighbour
cudaError_t launch_count_obstacle_nodes(const uint16_t *links, int W, int H, int P, unsigned long long *counts,
                                        cudaStream_t s);
cudaError_t launch_npol(int prec, int lay, const StepParams &p, dim3 grid, dim3 block, cudaStream_t s);
// debugMode's unfused step of nptl (linear = false, 2-D blocks) or lptl (linear = true, the block's
// thread count as a 1-D block): stream, observables, collide; F64_STRICT and F32_REF (k_debug.cu).
cudaError_t launch_debug_step(int prec, int lay, bool linear, const StepParams &p, dim3 block, cudaStream_t s);
// Rows of a 32-wide nsol block whose even step in the collision layout stages its stores.
constexpr int NSOL_STAGE_ROWS = 8;
cudaError_t launch_nsol(int prec, int lay, const StepParams &p, unsigned t, dim3 grid, dim3 block, cudaStream_t s);

// Set-up kernels (plbm_util.cu).
cudaError_t launch_links(const int8_t *flags, uint16_t *links, int W, int H, int P, cudaStream_t s);
cudaError_t launch_check_mask(const int8_t *mask, unsigned long long n, int *bad, cudaStream_t s);
cudaError_t launch_fill_lattice(void *lat, int prec, int lay, unsigned long long N, const double w[9], cudaStream_t s);
cudaError_t launch_fill_shifted(void *lat, int prec, int lay, int P, unsigned long long N, const double w[9], double a,
                                double g, cudaStream_t s);
cudaError_t launch_fill_halo(void *halo, int prec, int W, int H, int ncb, int nrb, const double w[9], cudaStream_t s);
// n entries of a shifted-form lattice (F32, F16S, BF16S, F16C) re-encoded in another shifted form
cudaError_t launch_convert_shifted(const void *src, int src_prec, void *dst, int dst_prec, unsigned long long n,
                                   int *status, cudaStream_t s);
cudaError_t launch_fill_results(double *rho, double *jx, double *jy, double *ja, unsigned long long n, cudaStream_t s);
// FP64 sums over fluid nodes of the result arrays: out3 = {sum rho, sum jx, sum jy}.
cudaError_t launch_reduce_results(const double *rho, const double *jx, const double *jy, const int8_t *flags,
                                  unsigned long long n, double *out3_dev, cudaStream_t s);
// FP64 sums over fluid nodes: out2 = {sum |j - j_prev|^2, sum |j|^2}; then j_prev = j.
cudaError_t launch_residual(const double *jx, const double *jy, double *jx_prev, double *jy_prev, const int8_t *flags,
                            unsigned long long n, double *out2_dev, cudaStream_t s);
// Equilibrium populations of the fields rho, jx, jy (device, W*H doubles) into lattice `lat`.
cudaError_t launch_set_equilibrium(void *lat, int prec, int lay, const StepParams &p, const double *rho,
                                   const double *jx, const double *jy, cudaStream_t s);
int max_threads_for(int alg, int prec, int lay);

}  // namespace plbm
