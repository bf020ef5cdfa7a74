// plbm_util.cu — set-up and reduction kernels: link masks, lattice/halo/result fills, and the
// FP64 mass/momentum reduction.
#include "plbm_device.cuh"
#include "plbm_launch.h"

namespace plbm {

// Packs, for every inner node, whether it is fluid (bit 4), which pull sources n - c_d are
// solid (bit d) and whether it lies on the domain's edge (LINK_EDGE).  flags: W*H int8 (0 fluid, 1 solid), row-major; links: P*H uint16.
__global__ void k_links(const int8_t *flags, uint16_t *links, int W, int H, int P)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= P || y >= H) return;
    uint16_t v = 0;
    if (x < W && flags[(size_t)y * W + x] == 0) {
        v = LINK_FLUID;
        for (int d = 0; d < 9; ++d) {
            if (d == 4) continue;
            const int sx = x - (d % 3 - 1), sy = y - (d / 3 - 1);
            if (sx < 0 || sx >= W || sy < 0 || sy >= H) continue;
            if (flags[(size_t)sy * W + sx] == 1) v |= (uint16_t)(1u << d);
        }
    }
    if (x == 0 || x == W - 1 || y == 0 || y == H - 1) v |= LINK_EDGE;
    links[(size_t)y * P + x] = v;
}

// *bad = 1 if any entry of a caller's mask is neither 0 (fluid) nor 1 (solid).
__global__ void k_check_mask(const int8_t *mask, unsigned long long n, int *bad)
{
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x)
        if (mask[i] != 0 && mask[i] != 1) { *bad = 1; return; }
}

cudaError_t launch_check_mask(const int8_t *mask, unsigned long long n, int *bad, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    k_check_mask<<<152 * 8, 256, 0, s>>>(mask, n, bad);
    return cudaGetLastError();
}

cudaError_t launch_links(const int8_t *flags, uint16_t *links, int W, int H, int P, cudaStream_t s)
{
    dim3 grid((P + 255) / 256, H);
    k_links<<<grid, 256, 0, s>>>(flags, links, W, H, P);
    return cudaGetLastError();
}

// Over the 32-node row segments (P is a multiple of 32, so a warp's 32 consecutive nodes are one
// segment): counts[0] += segments holding fluid, counts[1] += segments whose interior fluid nodes
// mix both kinds, all sources fluid and some source solid (a warp that splits between gathers).
__global__ void k_count_obstacle_nodes(const uint16_t *links, int W, int H, int P, unsigned long long *counts)
{
    unsigned seg = 0, mixed = 0;
    const unsigned long long n = (unsigned long long)P * H;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;   // a multiple of 32
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint16_t lk = links[i];   // the loop bound is warp-uniform: n is a multiple of 32
        const unsigned fl = __ballot_sync(0xffffffffu, (lk & LINK_FLUID) != 0);
        const unsigned plain = __ballot_sync(0xffffffffu, lk == LINK_FLUID);
        const unsigned near = __ballot_sync(0xffffffffu, (lk & (LINK_FLUID | LINK_EDGE)) == LINK_FLUID && lk != LINK_FLUID);
        seg += fl != 0;
        mixed += plain != 0 && near != 0;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&counts[0], (unsigned long long)seg);
        atomicAdd(&counts[1], (unsigned long long)mixed);
    }
    (void)W;
}

cudaError_t launch_count_obstacle_nodes(const uint16_t *links, int W, int H, int P, unsigned long long *counts,
                                        cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(counts, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    k_count_obstacle_nodes<<<152 * 4, 256, 0, s>>>(links, W, H, P, counts);
    return cudaGetLastError();
}

struct W9 { double w[9]; };

template <int PREC>
__global__ void k_fill_lattice(void *lat, int lay, unsigned long long N, W9 w)
{
    using T = typename Store<PREC>::T;
    const unsigned long long total = 9ull * N;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        int d;
        if (lay == COLLISION) d = (int)(i % 9);
        else if (lay == STREAM) d = (int)(i / N);
        else d = 3 * (int)(i / (3 * N)) + (int)((i % (3 * N)) % 3);
        T *b = static_cast<T *>(lat);
        if constexpr (PREC == F64_Q60) b[i] = double_to_q(w.w[d]);
        else if constexpr (PREC == F16S) b[i] = __float2half_rn(0.0f);
        else if constexpr (PREC == BF16S) b[i] = __float2bfloat16_rn(0.0f);
        else if constexpr (PREC == F16C) b[i] = 0;
        else b[i] = (T)w.w[d];
    }
}

cudaError_t launch_fill_lattice(void *lat, int prec, int lay, unsigned long long N, const double w[9], cudaStream_t s)
{
    W9 ww;
    for (int i = 0; i < 9; ++i) ww.w[i] = w[i];
    const int grid = 152 * 8, block = 256;
    switch (prec) {
    case F64_STRICT: case F64_FAST: k_fill_lattice<F64_STRICT><<<grid, block, 0, s>>>(lat, lay, N, ww); break;
    case F32_REF: case F32: k_fill_lattice<F32><<<grid, block, 0, s>>>(lat, lay, N, ww); break;
    case F16S: k_fill_lattice<F16S><<<grid, block, 0, s>>>(lat, lay, N, ww); break;
    case BF16S: k_fill_lattice<BF16S><<<grid, block, 0, s>>>(lat, lay, N, ww); break;
    case F16C: k_fill_lattice<F16C><<<grid, block, 0, s>>>(lat, lay, N, ww); break;
    case F64_Q60: k_fill_lattice<F64_Q60><<<grid, block, 0, s>>>(lat, lay, N, ww); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// Shifted forms: the rest state (rho = 1, j = 0) as deviations from w_d * rho0(x'),
// rho0(x') = a - g x', i.e. w_d ((1 - a) + g x').
template <int PREC>
__global__ void k_fill_shifted(void *lat, int lay, int P, unsigned long long N, W9 w, double a, double g)
{
    const unsigned long long total = 9ull * N;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        int d;
        unsigned long long n;
        if (lay == COLLISION) { d = (int)(i % 9); n = i / 9; }
        else if (lay == STREAM) { d = (int)(i / N); n = i % N; }
        else { const unsigned long long r = i % (3 * N); d = 3 * (int)(i / (3 * N)) + (int)(r % 3); n = r / 3; }
        const int x = (int)(n % (unsigned long long)P);
        const float v = (float)(w.w[d] * ((1.0 - a) + g * x));
        if constexpr (PREC == F16S) static_cast<__half *>(lat)[i] = __float2half_rn(v * F16_SCALE);
        else if constexpr (PREC == BF16S) static_cast<__nv_bfloat16 *>(lat)[i] = __float2bfloat16_rn(v);
        else if constexpr (PREC == F16C) {
            bool over;   // the host admits the form only where the rest state's deviations fit
            static_cast<unsigned short *>(lat)[i] = (unsigned short)f16c_bits(v, over);
        } else static_cast<float *>(lat)[i] = v;
    }
}

cudaError_t launch_fill_shifted(void *lat, int prec, int lay, int P, unsigned long long N, const double w[9], double a,
                                double g, cudaStream_t s)
{
    W9 ww;
    for (int i = 0; i < 9; ++i) ww.w[i] = w[i];
    const int grid = 152 * 8, block = 256;
    switch (prec) {
    case F32: k_fill_shifted<F32><<<grid, block, 0, s>>>(lat, lay, P, N, ww, a, g); break;
    case F16S: k_fill_shifted<F16S><<<grid, block, 0, s>>>(lat, lay, P, N, ww, a, g); break;
    case BF16S: k_fill_shifted<BF16S><<<grid, block, 0, s>>>(lat, lay, P, N, ww, a, g); break;
    case F16C: k_fill_shifted<F16C><<<grid, block, 0, s>>>(lat, lay, P, N, ww, a, g); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// A lattice or halo snapshot of one shifted storage form re-encoded in another.  Both hold the
// deviation df = f - w_d rho0(x') from the same reference state (the FP16 form scaled by F16_SCALE,
// a power of two): the value is decoded to FP32, rescaled exactly and rounded once into the new
// form; a value beyond the F16C range sets bit 0 of *status.
template <int SRC, int DST>
__global__ void k_convert_shifted(const void *src, void *dst, unsigned long long n, int *status)
{
    using TS = typename Store<SRC>::T;
    using TD = typename Store<DST>::T;
    bool over = false;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const TS s = static_cast<const TS *>(src)[i];
        float v;
        if constexpr (SRC == F16S) v = __half2float(s) * (1.0f / F16_SCALE);
        else if constexpr (SRC == BF16S) v = __bfloat162float(s);
        else if constexpr (SRC == F16C) v = f16c_value(s);
        else v = s;
        TD *d = static_cast<TD *>(dst);
        if constexpr (DST == F16S) d[i] = __float2half_rn(v * F16_SCALE);
        else if constexpr (DST == BF16S) d[i] = __float2bfloat16_rn(v);
        else if constexpr (DST == F16C) {
            bool o;
            d[i] = (unsigned short)f16c_bits(v, o);
            over |= o;
        } else d[i] = v;
    }
    if (over) atomicOr(status, 1);
}

template <int SRC>
static cudaError_t convert_from(const void *src, int dst_prec, void *dst, unsigned long long n, int *status,
                                cudaStream_t s)
{
    const int grid = 152 * 8, block = 256;
    switch (dst_prec) {
    case F32: k_convert_shifted<SRC, F32><<<grid, block, 0, s>>>(src, dst, n, status); break;
    case F16S: k_convert_shifted<SRC, F16S><<<grid, block, 0, s>>>(src, dst, n, status); break;
    case BF16S: k_convert_shifted<SRC, BF16S><<<grid, block, 0, s>>>(src, dst, n, status); break;
    case F16C: k_convert_shifted<SRC, F16C><<<grid, block, 0, s>>>(src, dst, n, status); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_convert_shifted(const void *src, int src_prec, void *dst, int dst_prec, unsigned long long n,
                                   int *status, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    switch (src_prec) {
    case F32: return convert_from<F32>(src, dst_prec, dst, n, status, s);
    case F16S: return convert_from<F16S>(src, dst_prec, dst, n, status, s);
    case BF16S: return convert_from<BF16S>(src, dst_prec, dst, n, status, s);
    case F16C: return convert_from<F16C>(src, dst_prec, dst, n, status, s);
    default: return cudaErrorInvalidValue;
    }
}

// Halo snapshot entries hold the rest state initially (w_d, or 0 for the shifted forms, whose
// npol lattice stores f - w_d); the direction of each slot follows the layout documented at k_npol.
template <int PREC>
__global__ void k_fill_halo(void *halo, unsigned long long ncol, unsigned long long total, int W, int H, W9 w)
{
    using T = typename Store<PREC>::T;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        // slot k of the [b][k][line] layout (halo_col / halo_row in plbm_kernels.cuh)
        int k, d;
        if (i < ncol) {
            k = (int)((i / (unsigned long long)H) % 6);
            d = k < 3 ? 3 * k + 2 : 3 * (k - 3);
        } else {
            k = (int)(((i - ncol) / (unsigned long long)W) % 6);
            d = k < 3 ? 6 + k : k - 3;
        }
        T *b = static_cast<T *>(halo);
        if constexpr (PREC == F64_Q60) b[i] = double_to_q(w.w[d]);
        else if constexpr (PREC == F16S) b[i] = __float2half_rn(0.0f);
        else if constexpr (PREC == BF16S) b[i] = __float2bfloat16_rn(0.0f);
        else if constexpr (PREC == F16C) b[i] = 0;
        else if constexpr (PREC == F32) b[i] = 0.0f;
        else b[i] = (T)w.w[d];
    }
}

cudaError_t launch_fill_halo(void *halo, int prec, int W, int H, int ncb, int nrb, const double w[9], cudaStream_t s)
{
    W9 ww;
    for (int i = 0; i < 9; ++i) ww.w[i] = w[i];
    const unsigned long long ncol = (unsigned long long)ncb * H * 6, total = ncol + (unsigned long long)nrb * W * 6;
    if (total == 0) return cudaSuccess;
    const int grid = 152 * 2, block = 256;
    switch (prec) {
    case F64_STRICT: case F64_FAST: k_fill_halo<F64_STRICT><<<grid, block, 0, s>>>(halo, ncol, total, W, H, ww); break;
    case F32_REF: k_fill_halo<F32_REF><<<grid, block, 0, s>>>(halo, ncol, total, W, H, ww); break;
    case F32: k_fill_halo<F32><<<grid, block, 0, s>>>(halo, ncol, total, W, H, ww); break;
    case F16S: k_fill_halo<F16S><<<grid, block, 0, s>>>(halo, ncol, total, W, H, ww); break;
    case BF16S: k_fill_halo<BF16S><<<grid, block, 0, s>>>(halo, ncol, total, W, H, ww); break;
    case F16C: k_fill_halo<F16C><<<grid, block, 0, s>>>(halo, ncol, total, W, H, ww); break;
    case F64_Q60: k_fill_halo<F64_Q60><<<grid, block, 0, s>>>(halo, ncol, total, W, H, ww); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// core::Results starts as if every node were solid: rho = -1, j = 0 (simulation.cpp:386-417).
__global__ void k_fill_results(double *rho, double *jx, double *jy, double *ja, unsigned long long n)
{
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        rho[i] = -1.0; jx[i] = 0.0; jy[i] = 0.0; ja[i] = 0.0;
    }
}

cudaError_t launch_fill_results(double *rho, double *jx, double *jy, double *ja, unsigned long long n, cudaStream_t s)
{
    k_fill_results<<<152 * 4, 256, 0, s>>>(rho, jx, jy, ja, n);
    return cudaGetLastError();
}

// Block-wise FP64 sums, then one atomicAdd per block and quantity.
__global__ void k_reduce_results(const double *rho, const double *jx, const double *jy, const int8_t *flags,
                                 unsigned long long n, double *out)
{
    double a = 0, b = 0, c = 0;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        if (flags[i] == 0) { a += rho[i]; b += jx[i]; c += jy[i]; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
    }
    __shared__ double sm[3][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { sm[0][wid] = a; sm[1][wid] = b; sm[2][wid] = c; }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        a = lane < nw ? sm[0][lane] : 0; b = lane < nw ? sm[1][lane] : 0; c = lane < nw ? sm[2][lane] : 0;
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
            c += __shfl_down_sync(0xffffffffu, c, o);
        }
        if (lane == 0) { atomicAdd(&out[0], a); atomicAdd(&out[1], b); atomicAdd(&out[2], c); }
    }
}

cudaError_t launch_reduce_results(const double *rho, const double *jx, const double *jy, const int8_t *flags,
                                  unsigned long long n, double *out3, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(out3, 0, 3 * sizeof(double), s);
    if (e != cudaSuccess) return e;
    k_reduce_results<<<152 * 2, 256, 0, s>>>(rho, jx, jy, flags, n, out3);
    return cudaGetLastError();
}

__global__ void k_residual(const double *jx, const double *jy, double *jxp, double *jyp, const int8_t *flags,
                           unsigned long long n, double *out)
{
    double a = 0, b = 0;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        if (flags[i] != 0) continue;
        const double x = jx[i], y = jy[i], dx = x - jxp[i], dy = y - jyp[i];
        a += dx * dx + dy * dy;
        b += x * x + y * y;
        jxp[i] = x;
        jyp[i] = y;
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    __shared__ double sm[2][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { sm[0][wid] = a; sm[1][wid] = b; }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        a = lane < nw ? sm[0][lane] : 0;
        b = lane < nw ? sm[1][lane] : 0;
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
        }
        if (lane == 0) { atomicAdd(&out[0], a); atomicAdd(&out[1], b); }
    }
}

cudaError_t launch_residual(const double *jx, const double *jy, double *jx_prev, double *jy_prev, const int8_t *flags,
                            unsigned long long n, double *out2, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(out2, 0, 2 * sizeof(double), s);
    if (e != cudaSuccess) return e;
    k_residual<<<152 * 2, 256, 0, s>>>(jx, jy, jx_prev, jy_prev, flags, n, out2);
    return cudaGetLastError();
}

template <int PREC, int L>
__global__ void k_set_equilibrium(void *lat, StepParams p, const double *rho, const double *jx, const double *jy)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= p.W || y >= p.H) return;
    const size_t r = (size_t)y * p.W + x;
    const unsigned long long n = (unsigned long long)x + (unsigned long long)y * p.P;
    // solid nodes get the rest state, as at initialisation (their populations are never read)
    const bool fluid = (p.links[n] & LINK_FLUID) != 0;
    const double R = fluid ? rho[r] : 1.0, X = fluid ? jx[r] : 0.0, Y = fluid ? jy[r] : 0.0, usq = X * X + Y * Y;
    for (int d = 0; d < 9; ++d) {
        const double cu = (d % 3 - 1) * X + (d / 3 - 1) * Y;
        const double w = p.weight[d];
        const double f = w * (R + 3 * cu + 4.5 * cu * cu - 1.5 * usq);
        typename Store<PREC>::C v;
        if constexpr (PREC == F64_Q60) v = double_to_q(f);
        else if constexpr (PREC == F16S) v = (float)((f - w * (p.shift_a - p.shift_g * x)) * F16_SCALE);
        else if constexpr (shifted<PREC>()) v = (float)(f - w * (p.shift_a - p.shift_g * x));
        else v = (typename Store<PREC>::C)f;
        st<PREC>(lat, lidx<L>(n, d, p.N), d, v, p);
    }
}

cudaError_t launch_set_equilibrium(void *lat, int prec, int lay, const StepParams &p, const double *rho,
                                   const double *jx, const double *jy, cudaStream_t s)
{
    const dim3 grid((p.W + 127) / 128, p.H), block(128);
#define PLBM_EQ(PR)                                                                                       \
    case PR:                                                                                              \
        if (lay == COLLISION) k_set_equilibrium<PR, COLLISION><<<grid, block, 0, s>>>(lat, p, rho, jx, jy); \
        else if (lay == STREAM) k_set_equilibrium<PR, STREAM><<<grid, block, 0, s>>>(lat, p, rho, jx, jy);  \
        else k_set_equilibrium<PR, BUNDLE><<<grid, block, 0, s>>>(lat, p, rho, jx, jy);                   \
        break;
    switch (prec) {
        PLBM_EQ(F64_STRICT) PLBM_EQ(F64_FAST) PLBM_EQ(F32_REF) PLBM_EQ(F32) PLBM_EQ(F16S) PLBM_EQ(BF16S) PLBM_EQ(F64_Q60) PLBM_EQ(F16C)
    default: return cudaErrorInvalidValue;
    }
#undef PLBM_EQ
    return cudaGetLastError();
}

}  // namespace plbm
