// plbm_noalloc.cu — plbm_nptl_steps_noalloc: the nptl step (FP64 drop-in form, stream layout)
// on caller-owned device buffers, with no device memory allocated by the library.
//
// Who needs it: host applications that own all device memory through their own allocator or
// arena and do not let a library allocate behind their back, and callers on a latency-critical
// path where cudaMalloc / cudaFree (which may synchronise the device) are not acceptable.  They
// pass the two lattices, the flag grid and the result arrays; the only other state the step
// needs — the outlet's jy column of the previous step, two parities — lives in the fixed device
// array below.
#include "../../include/plbm_c.h"
#include "plbm_kernels.cuh"
#include "plbm_launch.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

namespace {

constexpr unsigned NOALLOC_MAX_ROWS = PLBM_NOALLOC_MAX_ROWS;
constexpr int NOALLOC_MAX_DEVICES = 64;
// widest accepted row: the row pitch (inner_w rounded up to 32) and the grid stay within int
constexpr unsigned NOALLOC_MAX_WIDTH = 1u << 30;

// The scratch: jy at x' = W-2 for two step parities.  Every GPU that loads the library holds it
// (1 MiB) until the process exits; all calls share it.
static __device__ __align__(256) double g_noalloc_scratch[2 * NOALLOC_MAX_ROWS];

std::mutex g_mu;
double *g_scratch_addr[NOALLOC_MAX_DEVICES] = {};
thread_local char g_err[256];

// Solid-source bits are derived from the caller's flag grid on the fly (no link array).  One rule
// for both uses of a flag: 0 is fluid, any other value solid (a node that does not update is also
// a bounce-back source for its neighbours).
__global__ void k_nptl_noalloc(plbm::StepParams p, const int8_t *flags)
{
    using namespace plbm;
    const int xi = blockIdx.x * blockDim.x + threadIdx.x;
    const int yi = blockIdx.y * blockDim.y + threadIdx.y;
    if (xi >= p.W || yi >= p.H) return;
    if (flags[(size_t)yi * p.W + xi] != 0) return;
    uint16_t lk = LINK_FLUID;
#pragma unroll
    for (int d = 0; d < 9; ++d) {
        if (d == 4) continue;
        const int sx = xi - cxd(d), sy = yi - cyd(d);
        if (sx >= 0 && sx < p.W && sy >= 0 && sy < p.H && flags[(size_t)sy * p.W + sx] != 0) lk |= (uint16_t)(1u << d);
    }
    const unsigned long long n = (unsigned long long)xi + (unsigned long long)yi * p.P;
    double f[9];
#pragma unroll
    for (int d = 0; d < 9; ++d) f[d] = pull_one<F64_STRICT, STREAM>(p.lat0, n, xi, yi, d, lk, p);
    if (is_outlet_row(xi, yi, p)) outlet_fill<F64_STRICT>(f, jy_prev_at(p, yi), p);
    const Moments m = collide<F64_STRICT>(f, p);
#pragma unroll
    for (int d = 0; d < 9; ++d) st<F64_STRICT>(p.lat1, lidx<STREAM>(n, d, p.N), d, f[d], p);
    observables<F64_STRICT>(m, xi, yi, p);
}

__global__ void k_noalloc_clear(double *scratch, unsigned n)
{
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) scratch[i] = 0.0;
}

void mb(double ux, double uy, double rho, double *t)
{
    static const double w[9] = { 1.0 / 36, 1.0 / 9, 1.0 / 36, 1.0 / 9, 4.0 / 9, 1.0 / 9, 1.0 / 36, 1.0 / 9, 1.0 / 36 };
    for (int d = 0; d < 9; ++d) {
        const int vx = (d % 3) - 1, vy = (d / 3) - 1;
        t[d] = w[d] * (rho + 3 * (vx * ux + vy * uy) + 9.0 / 2 * std::pow(vx * ux + vy * uy, 2) -
                       3.0 / 2 * (ux * ux + uy * uy));
    }
}

int fail(int code, const char *msg)
{
    std::snprintf(g_err, sizeof g_err, "%s", msg);
    return code;
}

}  // namespace

extern "C" const char *plbm_noalloc_last_error(void) { return g_err; }

extern "C" int plbm_nptl_steps_noalloc(const plbm_noalloc_args *a)
{
    if (!a || !a->lattice0 || !a->lattice1 || !a->flags || !a->results)
        return fail(PLBM_ERR_ARGUMENT, "plbm_nptl_steps_noalloc: NULL buffer");
    if (a->inner_w < 2 || a->inner_h < 2) return fail(PLBM_ERR_ARGUMENT, "plbm_nptl_steps_noalloc: inner extents must be >= 2");
    if (a->inner_h > NOALLOC_MAX_ROWS)
        return fail(PLBM_ERR_ARGUMENT, "plbm_nptl_steps_noalloc: inner_h exceeds PLBM_NOALLOC_MAX_ROWS (65536)");
    if (a->inner_w > NOALLOC_MAX_WIDTH)
        return fail(PLBM_ERR_ARGUMENT, "plbm_nptl_steps_noalloc: inner_w exceeds 2^30 nodes");
    {
        // an error left pending by the caller's own earlier work is reported, not consumed: the
        // launch check below would otherwise return (and clear) it as this call's failure
        const cudaError_t pending = cudaPeekAtLastError();
        if (pending != cudaSuccess) {
            char msg[200];
            std::snprintf(msg, sizeof msg, "plbm_nptl_steps_noalloc: a CUDA error was already pending before the "
                                           "call (not cleared): %s", cudaGetErrorString(pending));
            return fail(PLBM_ERR_CUDA, msg);
        }
    }
    if (!(a->relaxation_time > 0)) return fail(PLBM_ERR_PROPERTY, "relaxation_time must be > 0");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return fail(PLBM_ERR_NO_DEVICE, "plbm_nptl_steps_noalloc: no current CUDA device");
    double *scratch = nullptr;
    {
        // Set-up on the first call on this device (the device must be current): the host-side
        // name of the __device__ array is not a device address, so fetch the real one once.
        std::lock_guard<std::mutex> g(g_mu);
        if (!g_scratch_addr[dev]) {
            void *ptr = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess) return fail(PLBM_ERR_CUDA, cudaGetErrorString(e));
            g_scratch_addr[dev] = static_cast<double *>(ptr);
        }
        scratch = g_scratch_addr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(a->stream);
    const int W = (int)a->inner_w, H = (int)a->inner_h, P = (W + 31) / 32 * 32;
    const unsigned long long N = (unsigned long long)P * H, nres = (unsigned long long)W * H;

    plbm::StepParams p;
    std::memset(&p, 0, sizeof p);
    mb(0, 0, 1, p.weight);
    mb(a->inlet_velocity_x, a->inlet_velocity_y, a->inlet_density, p.feq_in);
    mb(a->outlet_velocity_x, a->outlet_velocity_y, a->outlet_density, p.feq_out);
    p.omega = 1 / a->relaxation_time;
    p.rho_out = a->outlet_density;
    p.W = W; p.H = H; p.P = P; p.N = N;
    p.lat_elems = 9ull * N;
    p.nan_protection = a->nan_protection;
    double *res = static_cast<double *>(a->results);
    p.rho = res; p.jx = res + nres; p.jy = res + 2 * nres; p.jabs = res + 3 * nres;
    cudaError_t e = cudaSuccess;
    if (a->first_step == 0) {
        // A run starts from the rest state; the jy column of "step -1" is zero.
        e = plbm::launch_fill_lattice(a->lattice0, PLBM_F64_STRICT, plbm::STREAM, N, p.weight, s);
        if (e == cudaSuccess) e = plbm::launch_fill_lattice(a->lattice1, PLBM_F64_STRICT, plbm::STREAM, N, p.weight, s);
        if (e == cudaSuccess) e = plbm::launch_fill_results(p.rho, p.jx, p.jy, p.jabs, nres, s);
        if (e == cudaSuccess) {
            k_noalloc_clear<<<64, 256, 0, s>>>(scratch, 2 * (unsigned)H);
            e = cudaGetLastError();
        }
    }
    const dim3 block(32, 8), grid((W + 31) / 32, (H + 7) / 8);
    void *lat[2] = { a->lattice0, a->lattice1 };
    for (unsigned k = 0; k < a->steps && e == cudaSuccess; ++k) {
        const unsigned t = a->first_step + k, par = t & 1u;
        p.lat0 = lat[par];
        p.lat1 = lat[par ^ 1u];
        p.jy_prev = scratch + (size_t)par * H;
        p.jy_next = scratch + (size_t)(par ^ 1u) * H;
        p.write_results = (k + 1 == a->steps);
        k_nptl_noalloc<<<grid, block, 0, s>>>(p, a->flags);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return fail(PLBM_ERR_CUDA, cudaGetErrorString(e));
    return PLBM_OK;
}
