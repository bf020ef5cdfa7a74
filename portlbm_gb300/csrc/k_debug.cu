// k_debug.cu — the unfused timestep that debugMode selects for the two-lattice algorithms.
//
// With debugMode the reference's NPTLDebug / LPTLDebug drivers (nptl.hpp:166-514,
// lptl.hpp:168-517) replace the fused StreamCollideKernel by three kernels per step:
//   StreamKernel                   pull the nine incoming populations into lattice 1
//                                  (nptl_kernels.hpp:49-97, lptl_kernels.hpp:51-95)
//   MacroscopicObservablesKernel   rho, j, |j| of lattice 1 into the result arrays, NaN-guarded
//                                  (nptl_kernels.hpp:105-207)
//   CollideKernel                  BGK relaxation of lattice 1 in place, the equilibrium taken
//                                  from the stored (guarded) results (nptl_kernels.hpp:215-295)
// The same three launches run here, in the reference's operation order, for the FP64 drop-in
// (F64_STRICT) and the USE_FLOAT form (F32_REF); results equal the fused step's bit for bit
// whenever no observable is NaN or beyond FLT_MAX.  npol / nsol keep the fused kernel in debug
// mode, as the reference's NPOLDebug / NSOLDebug do.  The reference's console dumps are not
// reproduced.  Bounce-back, ghost and outlet values enter through the stream kernel's gather.
#include "plbm_kernels.cuh"
#include "plbm_launch.h"

namespace plbm {

// Node of this thread: 2-D grid over the inner W x H nodes (nptl) or 1-D over n = x' + y' * P
// (lptl, padding columns skipped).
template <bool LINEAR>
__device__ __forceinline__ bool debug_node(const StepParams &p, int &xi, int &yi, unsigned long long &n)
{
    if (LINEAR) {
        n = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
        if (n >= p.N) return false;
        yi = (int)(n / (unsigned)p.P);
        xi = (int)(n - (unsigned long long)yi * p.P);
        return xi < p.W;
    }
    xi = blockIdx.x * blockDim.x + threadIdx.x;
    yi = blockIdx.y * blockDim.y + threadIdx.y;
    n = (unsigned long long)xi + (unsigned long long)yi * p.P;
    return xi < p.W && yi < p.H;
}

template <int PREC, int L, bool LINEAR>
__global__ void k_debug_stream(StepParams p)
{
    int xi, yi;
    unsigned long long n;
    if (!debug_node<LINEAR>(p, xi, yi, n)) return;
    const uint16_t lk = link_at(p, n);
    if (!(lk & LINK_FLUID)) return;
    CT<PREC> f[9];
#pragma unroll
    for (int d = 0; d < 9; ++d) f[d] = pull_one<PREC, L>(p.lat0, n, xi, yi, d, lk, p);
    if (is_outlet_row(xi, yi, p)) outlet_fill<PREC>(f, jy_prev_at(p, yi), p);
#pragma unroll
    for (int d = 0; d < 9; ++d) st<PREC>(p.lat1, lidx<L>(n, d, p.N), d, f[d], p);
}

// Moments summed in direction order 0..8 (rho += f_d, j += f_d c_d), every operation rounded.
template <typename R>
__device__ __forceinline__ void debug_moments(const R f[9], R &rho, R &jx, R &jy)
{
    if constexpr (sizeof(R) == 8) {
        rho = f[0];
        for (int d = 1; d < 9; ++d) rho = __dadd_rn(rho, f[d]);
        jx = __dadd_rn(-f[0], f[2]);
        jx = __dsub_rn(jx, f[3]); jx = __dadd_rn(jx, f[5]); jx = __dsub_rn(jx, f[6]); jx = __dadd_rn(jx, f[8]);
        jy = __dsub_rn(-f[0], f[1]);
        jy = __dsub_rn(jy, f[2]); jy = __dadd_rn(jy, f[6]); jy = __dadd_rn(jy, f[7]); jy = __dadd_rn(jy, f[8]);
    } else {
        rho = f[0];
        for (int d = 1; d < 9; ++d) rho = __fadd_rn(rho, f[d]);
        jx = __fadd_rn(-f[0], f[2]);
        jx = __fsub_rn(jx, f[3]); jx = __fadd_rn(jx, f[5]); jx = __fsub_rn(jx, f[6]); jx = __fadd_rn(jx, f[8]);
        jy = __fsub_rn(-f[0], f[1]);
        jy = __fsub_rn(jy, f[2]); jy = __fadd_rn(jy, f[6]); jy = __fadd_rn(jy, f[7]); jy = __fadd_rn(jy, f[8]);
    }
}

// NaN protection of the USE_FLOAT build compares floats with FLT_MAX; the double form compares
// doubles with FLT_MAX (nan_guard).
__device__ __forceinline__ float nan_guard_f(float v) { return (isnan(v) || v > 3.4028234663852886e38f) ? 0.0f : v; }

template <int PREC, int L, bool LINEAR>
__global__ void k_debug_observables(StepParams p)
{
    int xi, yi;
    unsigned long long n;
    if (!debug_node<LINEAR>(p, xi, yi, n)) return;
    if (!(link_at(p, n) & LINK_FLUID)) return;
    using R = CT<PREC>;
    R f[9];
#pragma unroll
    for (int d = 0; d < 9; ++d) f[d] = ld<PREC>(p.lat1, lidx<L>(n, d, p.N), d, p);
    R rho, jx, jy, ja;
    debug_moments<R>(f, rho, jx, jy);
    if constexpr (sizeof(R) == 8) {
        ja = sqrt(__dadd_rn(__dmul_rn(jx, jx), __dmul_rn(jy, jy)));
        if (p.nan_protection) { rho = nan_guard(rho); jx = nan_guard(jx); jy = nan_guard(jy); ja = nan_guard(ja); }
    } else {
        ja = sqrtf(__fadd_rn(__fmul_rn(jx, jx), __fmul_rn(jy, jy)));
        if (p.nan_protection) { rho = nan_guard_f(rho); jx = nan_guard_f(jx); jy = nan_guard_f(jy); ja = nan_guard_f(ja); }
    }
    const unsigned long long r = (unsigned long long)xi + (unsigned long long)yi * p.W;
    if (!in_range(r, (unsigned long long)p.W * p.H, p)) return;
    p.rho[r] = rho; p.jx[r] = jx; p.jy[r] = jy; p.jabs[r] = ja;
    // the outlet reads this step's jy of column W-2 (the reference reads the result array)
    if (xi == p.W - 2 && p.jy_next && in_range((unsigned long long)yi, (unsigned long long)p.H, p)) p.jy_next[yi] = jy;
}

template <int PREC, int L, bool LINEAR>
__global__ void k_debug_collide(StepParams p)
{
    int xi, yi;
    unsigned long long n;
    if (!debug_node<LINEAR>(p, xi, yi, n)) return;
    if (!(link_at(p, n) & LINK_FLUID)) return;
    const unsigned long long r = (unsigned long long)xi + (unsigned long long)yi * p.W;
    // lidx(n, 0) and lidx(n, 8) bound the node's nine entries in every layout
    if (!in_range(r, (unsigned long long)p.W * p.H, p) || !in_range(lidx<L>(n, 8, p.N), p.lat_elems, p) ||
        !in_range(lidx<L>(n, 0, p.N), p.lat_elems, p))
        return;
    if constexpr (PREC == F64_STRICT) {
        const double rho = p.rho[r], ux = p.jx[r], uy = p.jy[r];
        const double usq = __dadd_rn(__dmul_rn(ux, ux), __dmul_rn(uy, uy));
        const double nom = -p.omega;
#pragma unroll
        for (int d = 0; d < 9; ++d) {
            const unsigned long long i = lidx<L>(n, d, p.N);
            const double v = static_cast<const double *>(p.lat1)[i];
            const double cu = __dadd_rn(__dmul_rn((double)cxd(d), ux), __dmul_rn((double)cyd(d), uy));
            const double br = __dsub_rn(__dadd_rn(__dadd_rn(rho, __dmul_rn(3.0, cu)), __dmul_rn(__dmul_rn(4.5, cu), cu)),
                                        __dmul_rn(1.5, usq));
            const double feq = __dmul_rn(p.weight[d], br);
            static_cast<double *>(p.lat1)[i] = __dadd_rn(__dmul_rn(nom, __dsub_rn(v, feq)), v);
        }
    } else {
        // real_type float; the double literals 9.0/2 and 3.0/2 promote the bracket to double,
        // rounded to float when assigned (nptl_kernels.hpp:268-282)
        const float rho = (float)p.rho[r], ux = (float)p.jx[r], uy = (float)p.jy[r];
        const float usq = __fadd_rn(__fmul_rn(ux, ux), __fmul_rn(uy, uy));
        const float nom = -p.omegaf;
#pragma unroll
        for (int d = 0; d < 9; ++d) {
            const unsigned long long i = lidx<L>(n, d, p.N);
            const float v = static_cast<const float *>(p.lat1)[i];
            const float cu = __fadd_rn(__fmul_rn((float)cxd(d), ux), __fmul_rn((float)cyd(d), uy));
            const double br = __dsub_rn(__dadd_rn((double)__fadd_rn(rho, __fmul_rn(3.0f, cu)),
                                                  __dmul_rn(__dmul_rn(4.5, (double)cu), (double)cu)),
                                        __dmul_rn(1.5, (double)usq));
            const float feq = (float)__dmul_rn((double)(float)p.weight[d], br);
            static_cast<float *>(p.lat1)[i] = __fadd_rn(__fmul_rn(nom, __fsub_rn(v, feq)), v);
        }
    }
}

template <int PREC, int L, bool LINEAR>
static cudaError_t debug_step(const StepParams &p, dim3 grid, dim3 block, cudaStream_t s)
{
    k_debug_stream<PREC, L, LINEAR><<<grid, block, 0, s>>>(p);
    k_debug_observables<PREC, L, LINEAR><<<grid, block, 0, s>>>(p);
    k_debug_collide<PREC, L, LINEAR><<<grid, block, 0, s>>>(p);
    return cudaGetLastError();
}

template <int PREC, bool LINEAR>
static cudaError_t debug_step_layout(int lay, const StepParams &p, dim3 grid, dim3 block, cudaStream_t s)
{
    switch (lay) {
    case COLLISION: return debug_step<PREC, COLLISION, LINEAR>(p, grid, block, s);
    case STREAM: return debug_step<PREC, STREAM, LINEAR>(p, grid, block, s);
    case BUNDLE: return debug_step<PREC, BUNDLE, LINEAR>(p, grid, block, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_debug_step(int prec, int lay, bool linear, const StepParams &p, dim3 block, cudaStream_t s)
{
    dim3 grid;
    if (linear) {
        block = dim3(block.x * block.y * block.z);
        grid = dim3((unsigned)((p.N + block.x - 1) / block.x));
    } else {
        grid = dim3((p.W + block.x - 1) / block.x, (p.H + block.y - 1) / block.y);
    }
    if (prec == F64_STRICT) return linear ? debug_step_layout<F64_STRICT, true>(lay, p, grid, block, s)
                                          : debug_step_layout<F64_STRICT, false>(lay, p, grid, block, s);
    if (prec == F32_REF) return linear ? debug_step_layout<F32_REF, true>(lay, p, grid, block, s)
                                       : debug_step_layout<F32_REF, false>(lay, p, grid, block, s);
    return cudaErrorInvalidValue;
}

}  // namespace plbm
