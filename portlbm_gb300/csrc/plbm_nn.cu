// plbm_nn.cu — the convolutional neural operator's kernels: the dispatch of the 3x3 "same"
// convolutions (forward, data gradient, weight gradient) to the tcgen05 kernels of plbm_nn_tc.cu,
// with an implicit GEMM on mma.sync m16n8k16 (BF16, FP32 accumulate) for the shapes those do not
// tile; 2x2 average pooling, nearest upsampling, skip addition, ReLU backward, the masked MSE loss
// and Adam.  Activations are NHWC bfloat16; weights are
// W[co][k] with k = (ky * 3 + kx) * Cin + ci (bfloat16, FP32 master copy updated by Adam).
//
// No counterpart in the reference: this is the learned warm-start addition of the GB300 build.
#include "../../include/plbm_c.h"

#include <cuda_bf16.h>
#include <mutex>
#include <cuda_runtime.h>
#include <stdint.h>

// Tensor-core convolution (plbm_nn_tc.cu).
bool plbm_nn_tc_supported(int H, int W, int Cin, int Cout);
int plbm_nn_tc_conv(const void *x, const void *w, const float *bias, void *y, int N, int H, int W, int Cin, int Cout,
                    int relu, cudaStream_t s);
int plbm_nn_tc_flip(const void *w, void *wt, int Cin, int Cout, cudaStream_t s);
bool plbm_nn_tc_wgrad_supported(int H, int W, int Cin, int Cout);
int plbm_nn_tc_wgrad(const void *x, const void *g, float *gw, float *gb, int N, int H, int W, int Cin, int Cout,
                     int *bias_done, cudaStream_t s);
bool plbm_nn_tc_small_supported(int H, int W, int Cin, int Cout);
int plbm_nn_tc_small_conv(const void *x, const void *w, const float *bias, void *y, int N, int H, int W, int Cin,
                          int Cout, int relu, cudaStream_t s);
bool plbm_nn_tc_small_wgrad_supported(int H, int W, int Cin, int Cout);
int plbm_nn_tc_small_wgrad(const void *x, const void *g, float *gw, int N, int H, int W, int Cin, int Cout,
                           cudaStream_t s);

namespace {

constexpr int BM = 128, BN = 64, BK = 32, PAD = 8, THREADS = 256;

enum Mode { FWD = 0, DGRAD = 1, WGRAD = 2 };

struct ConvArgs {
    const __nv_bfloat16 *x;    // FWD/WGRAD: input [N,H,W,Cin]
    const __nv_bfloat16 *g;    // DGRAD/WGRAD: gradient of the output [N,H,W,Cout]
    const __nv_bfloat16 *w;    // [Cout][9*Cin]
    const float *bias;         // FWD: [Cout] or null
    __nv_bfloat16 *y;          // FWD: output; DGRAD: gradient of the input
    float *gw;                 // WGRAD: [Cout][9*Cin] accumulated (atomicAdd)
    int N, H, W, Cin, Cout, relu;
    int M, Ncols, K;           // GEMM sizes of the mode
    int k_chunk;               // WGRAD: pixels per block (split K)
};

__device__ __forceinline__ __nv_bfloat16 bzero() { return __float2bfloat16_rn(0.0f); }

// Element (m, k) of the GEMM's A operand and (n, k) of its B operand for each mode.
template <int MODE>
__device__ __forceinline__ __nv_bfloat16 load_a(const ConvArgs &a, int m, int k)
{
    if (m >= a.M || k >= a.K) return bzero();
    if (MODE == FWD || MODE == DGRAD) {
        const int C = MODE == FWD ? a.Cin : a.Cout;
        const int tap = k / C, c = k - tap * C, ky = tap / 3, kx = tap - ky * 3;
        const int x = m % a.W, t = m / a.W, yv = t % a.H, n = t / a.H;
        const int sy = MODE == FWD ? yv + ky - 1 : yv - ky + 1, sx = MODE == FWD ? x + kx - 1 : x - kx + 1;
        if (sy < 0 || sy >= a.H || sx < 0 || sx >= a.W) return bzero();
        const __nv_bfloat16 *src = MODE == FWD ? a.x : a.g;
        return src[(((size_t)n * a.H + sy) * a.W + sx) * C + c];
    } else {   // WGRAD: A[co][pixel] = g[pixel][co]
        return a.g[(size_t)k * a.Cout + m];
    }
}

template <int MODE>
__device__ __forceinline__ __nv_bfloat16 load_b(const ConvArgs &a, int ncol, int k)
{
    if (ncol >= a.Ncols || k >= a.K) return bzero();
    if (MODE == FWD) {
        return a.w[(size_t)ncol * (9 * a.Cin) + k];
    } else if (MODE == DGRAD) {   // B[ci][(tap, co)] = W[co][(tap, ci)]
        const int tap = k / a.Cout, co = k - tap * a.Cout;
        return a.w[(size_t)co * (9 * a.Cin) + tap * a.Cin + ncol];
    } else {   // WGRAD: B[(tap, ci)][pixel] = x[pixel + offset(tap)][ci]
        const int tap = ncol / a.Cin, ci = ncol - tap * a.Cin, ky = tap / 3, kx = tap - ky * 3;
        const int p = k, x = p % a.W, t = p / a.W, yv = t % a.H, n = t / a.H;
        const int sy = yv + ky - 1, sx = x + kx - 1;
        if (sy < 0 || sy >= a.H || sx < 0 || sx >= a.W) return bzero();
        return a.x[(((size_t)n * a.H + sy) * a.W + sx) * a.Cin + ci];
    }
}

__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], const uint32_t b[2])
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C[BM x BN] tile of block (blockIdx.x over M, blockIdx.y over N); WGRAD splits K over blockIdx.z.
template <int MODE>
__global__ void __launch_bounds__(THREADS) k_conv(ConvArgs a)
{
    __shared__ __align__(16) __nv_bfloat16 As[BM][BK + PAD];
    __shared__ __align__(16) __nv_bfloat16 Bs[BN][BK + PAD];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int wm = warp & 3, wn = warp >> 2;          // 4 x 2 warps, 32 x 32 each
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    int k_begin = 0, k_end = a.K;
    if (MODE == WGRAD) {
        k_begin = blockIdx.z * a.k_chunk;
        k_end = min(a.K, k_begin + a.k_chunk);
    }
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
    const int grp = lane >> 2, tig = lane & 3;
    for (int k0 = k_begin; k0 < k_end; k0 += BK) {
        for (int i = tid; i < BM * BK; i += THREADS) {
            const int r = i / BK, c = i % BK, k = k0 + c;
            As[r][c] = k < k_end ? load_a<MODE>(a, m0 + r, k) : bzero();
        }
        for (int i = tid; i < BN * BK; i += THREADS) {
            const int r = i / BK, c = i % BK, k = k0 + c;
            Bs[r][c] = k < k_end ? load_b<MODE>(a, n0 + r, k) : bzero();
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t af[2][4], bf[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = wm * 32 + i * 16 + grp;
                af[i][0] = *reinterpret_cast<const uint32_t *>(&As[r][kk + tig * 2]);
                af[i][1] = *reinterpret_cast<const uint32_t *>(&As[r + 8][kk + tig * 2]);
                af[i][2] = *reinterpret_cast<const uint32_t *>(&As[r][kk + tig * 2 + 8]);
                af[i][3] = *reinterpret_cast<const uint32_t *>(&As[r + 8][kk + tig * 2 + 8]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = wn * 32 + j * 8 + grp;
                bf[j][0] = *reinterpret_cast<const uint32_t *>(&Bs[c][kk + tig * 2]);
                bf[j][1] = *reinterpret_cast<const uint32_t *>(&Bs[c][kk + tig * 2 + 8]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma16816(acc[i][j], af[i], bf[j]);
        }
        __syncthreads();
    }
    // epilogue
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int m = m0 + wm * 32 + i * 16 + grp + (r >= 2 ? 8 : 0);
                const int n = n0 + wn * 32 + j * 8 + tig * 2 + (r & 1);
                if (m >= a.M || n >= a.Ncols) continue;
                float v = acc[i][j][r];
                if (MODE == FWD) {
                    if (a.bias) v += a.bias[n];
                    if (a.relu) v = fmaxf(v, 0.f);
                    a.y[(size_t)m * a.Cout + n] = __float2bfloat16_rn(v);
                } else if (MODE == DGRAD) {
                    a.y[(size_t)m * a.Cin + n] = __float2bfloat16_rn(v);
                } else {
                    atomicAdd(&a.gw[(size_t)m * (9 * a.Cin) + n], v);
                }
            }
}

__global__ void k_bias_grad(const __nv_bfloat16 *g, float *gb, long long P, int C)
{
    // one block per channel group of 32 channels x 8 pixel rows
    const int c = blockIdx.y * 32 + (threadIdx.x & 31);
    if (c >= C) return;
    float s = 0.f;
    for (long long p = blockIdx.x * 8 + (threadIdx.x >> 5); p < P; p += (long long)gridDim.x * 8)
        s += __bfloat162float(g[p * C + c]);
    atomicAdd(&gb[c], s);
}

__global__ void k_relu_bwd(const __nv_bfloat16 *y, __nv_bfloat16 *g, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        if (!(__bfloat162float(y[i]) > 0.f)) g[i] = __float2bfloat16_rn(0.f);
}

__global__ void k_pool2(const __nv_bfloat16 *x, __nv_bfloat16 *y, int N, int H, int W, int C)
{
    const int Ho = H / 2, Wo = W / 2;
    const long long total = (long long)N * Ho * Wo * C;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        long long t = i / C;
        const int xo = (int)(t % Wo); t /= Wo;
        const int yo = (int)(t % Ho);
        const int n = (int)(t / Ho);
        const size_t b = (((size_t)n * H + 2 * yo) * W + 2 * xo) * C + c;
        const float s = __bfloat162float(x[b]) + __bfloat162float(x[b + C]) + __bfloat162float(x[b + (size_t)W * C]) +
                        __bfloat162float(x[b + (size_t)W * C + C]);
        y[i] = __float2bfloat16_rn(0.25f * s);
    }
}

__global__ void k_pool2_bwd(const __nv_bfloat16 *gy, __nv_bfloat16 *gx, int N, int H, int W, int C)
{
    const long long total = (long long)N * H * W * C;
    const int Ho = H / 2, Wo = W / 2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        long long t = i / C;
        const int x = (int)(t % W); t /= W;
        const int yv = (int)(t % H);
        const int n = (int)(t / H);
        gx[i] = __float2bfloat16_rn(0.25f * __bfloat162float(gy[(((size_t)n * Ho + yv / 2) * Wo + x / 2) * C + c]));
    }
}

__global__ void k_up2(const __nv_bfloat16 *x, __nv_bfloat16 *y, int N, int H, int W, int C)   // H, W: output
{
    const long long total = (long long)N * H * W * C;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        long long t = i / C;
        const int xx = (int)(t % W); t /= W;
        const int yy = (int)(t % H);
        const int n = (int)(t / H);
        y[i] = x[(((size_t)n * (H / 2) + yy / 2) * (W / 2) + xx / 2) * C + c];
    }
}

__global__ void k_up2_bwd(const __nv_bfloat16 *gy, __nv_bfloat16 *gx, int N, int H, int W, int C)   // H, W: input
{
    const long long total = (long long)N * H * W * C;
    const int Ho = 2 * H, Wo = 2 * W;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        long long t = i / C;
        const int x = (int)(t % W); t /= W;
        const int yv = (int)(t % H);
        const int n = (int)(t / H);
        const size_t b = (((size_t)n * Ho + 2 * yv) * Wo + 2 * x) * C + c;
        gx[i] = __float2bfloat16_rn(__bfloat162float(gy[b]) + __bfloat162float(gy[b + C]) +
                                    __bfloat162float(gy[b + (size_t)Wo * C]) + __bfloat162float(gy[b + (size_t)Wo * C + C]));
    }
}

__global__ void k_add(const __nv_bfloat16 *a, const __nv_bfloat16 *b, __nv_bfloat16 *y, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = __float2bfloat16_rn(__bfloat162float(a[i]) + __bfloat162float(b[i]));
}

// Masked mean squared error over fluid pixels of C channels: loss += sum / count, grad = 2 (p - t) / count.
__global__ void k_mse(const __nv_bfloat16 *pred, const float *target, const int8_t *mask, __nv_bfloat16 *grad,
                      float *loss, long long P, int C, float inv_count)
{
    float s = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P * C; i += (long long)gridDim.x * blockDim.x) {
        const long long p = i / C;
        float gval = 0.f;
        if (mask[p] == 0) {
            const float d = __bfloat162float(pred[i]) - target[i];
            s += d * d;
            gval = 2.f * d * inv_count;
        }
        grad[i] = __float2bfloat16_rn(gval);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s * inv_count);
}

__global__ void k_adam(float *w, const float *g, float *m, float *v, __nv_bfloat16 *wb, long long n, float lr, float b1,
                       float b2, float eps, float c1, float c2)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        w[i] = wi;
        if (wb) wb[i] = __float2bfloat16_rn(wi);
    }
}

// Adam with its step count and learning rate on the device, for a launch captured into a CUDA
// graph: every block reads state[0] = t and updates with step t + 1; the last block to finish
// (state[1] counts finished blocks) stores t + 1 and clears the count, so each replay advances it.
__global__ void k_adam_dev(float *w, const float *g, float *m, float *v, __nv_bfloat16 *wb, long long n,
                           const float *lr_p, float b1, float b2, float eps, int *state)
{
    __shared__ bool last;
    const int t = state[0] + 1;
    const float lr = *lr_p;
    const float c1 = 1.f / (1.f - powf(b1, (float)t)), c2 = 1.f / (1.f - powf(b2, (float)t));
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        w[i] = wi;
        if (wb) wb[i] = __float2bfloat16_rn(wi);
    }
    __syncthreads();                       // every thread of the block has read state[0]
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd((unsigned int *)&state[1], 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        state[0] = t;
        state[1] = 0;
        __threadfence();
    }
}

// Network input: channel 0 fluid(0)/solid(1) mask, channels 1..3 the per-sample scalars
// features[n][0..2] as constant planes; channels beyond 4 are zero.
__global__ void k_assemble(const int8_t *mask, const float *features, __nv_bfloat16 *y, int N, int H, int W, int C)
{
    const long long total = (long long)N * H * W;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < total; p += (long long)gridDim.x * blockDim.x) {
        const int n = (int)(p / ((long long)H * W));
        const float v[4] = { (float)mask[p], features[3 * n], features[3 * n + 1], features[3 * n + 2] };
        for (int c = 0; c < C; ++c) y[p * C + c] = __float2bfloat16_rn(c < 4 ? v[c] : 0.f);
    }
}

// ---- 16-byte forms: eight channels per thread and 32-bit index arithmetic, for channel counts that
// are multiples of 8 (every layer of the operator but its 4-channel input and 3-channel output) ----
__device__ __forceinline__ void unpack8(const uint4 u, float f[8])
{
    const uint32_t w[4] = { u.x, u.y, u.z, u.w };
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        f[2 * k] = __uint_as_float(w[k] << 16);
        f[2 * k + 1] = __uint_as_float(w[k] & 0xffff0000u);
    }
}
__device__ __forceinline__ uint4 pack8(const float f[8])
{
    uint32_t w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        __nv_bfloat162 b = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
        w[k] = *reinterpret_cast<uint32_t *>(&b);
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

// Every layer's weights re-laid out for its input gradient in one launch: layer l = blockIdx.y,
// segs[3l..3l+2] = (element offset of its weights in the flat buffers, Cin, Cout);
// wt[off + (ci * 9 + 8 - tap) * Cout + co] = w[off + (co * 9 + tap) * Cin + ci].
__global__ void k_flip_layers(const __nv_bfloat16 *w, __nv_bfloat16 *wt, const int *segs)
{
    const long long off = segs[3 * blockIdx.y];
    const int Cin = segs[3 * blockIdx.y + 1], Cout = segs[3 * blockIdx.y + 2], total = Cout * 9 * Cin;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int co = i / (9 * Cin), r = i - co * 9 * Cin, tap = r / Cin, ci = r - tap * Cin;
        wt[off + ((long long)ci * 9 + (8 - tap)) * Cout + co] = w[off + i];
    }
}

// Eight bfloat16 gradients kept where y > 0 (a positive, non-NaN bfloat16), zeroed elsewhere.
__device__ __forceinline__ uint4 relu_mask8(uint4 yv, uint4 gv)
{
    uint32_t *gw = reinterpret_cast<uint32_t *>(&gv);
    const uint32_t yw[4] = { yv.x, yv.y, yv.z, yv.w };
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const bool lo = __uint_as_float(yw[k] << 16) > 0.f, hi = __uint_as_float(yw[k] & 0xffff0000u) > 0.f;
        gw[k] &= (lo ? 0x0000ffffu : 0u) | (hi ? 0xffff0000u : 0u);
    }
    return gv;
}

// gb[c] += sum over the P pixels of g[p][c]: thread (pixel lane q, unit u) of a block of
// R = blockDim.x / CU pixel lanes sums unit u of every (R * gridDim.x)-th pixel; the block's lanes
// are then added per channel in shared memory, one atomic per channel and block.  RELU: the ReLU
// backward first, in place (g = g * (y > 0)), and the masked values summed: one pass over g.
template <bool RELU>
__global__ void k_bias_grad_v(const uint4 *y, uint4 *g, float *gb, unsigned P, int CU)
{
    extern __shared__ float red[];
    const int R = blockDim.x / CU, q = threadIdx.x / CU, u = threadIdx.x - q * CU;
    float s[8] = { 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f };
    if (q < R)
        for (unsigned p = blockIdx.x * (unsigned)R + q; p < P; p += gridDim.x * (unsigned)R) {
            const size_t i = (size_t)p * CU + u;
            uint4 gv = g[i];
            if constexpr (RELU) {
                gv = relu_mask8(y[i], gv);
                g[i] = gv;
            }
            float f[8];
            unpack8(gv, f);
#pragma unroll
            for (int e = 0; e < 8; ++e) s[e] += f[e];
        }
    if (q < R)
#pragma unroll
        for (int e = 0; e < 8; ++e) red[threadIdx.x * 8 + e] = s[e];
    __syncthreads();
    for (int k = threadIdx.x; k < CU * 8; k += blockDim.x) {
        float t = 0.f;
        for (int qq = 0; qq < R; ++qq) t += red[qq * CU * 8 + k];
        atomicAdd(&gb[k], t);
    }
}

__global__ void k_relu_bwd_v(const uint4 *y, uint4 *g, unsigned n8)
{
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n8; i += gridDim.x * blockDim.x) g[i] = relu_mask8(y[i], g[i]);
}

__global__ void k_add_v(const uint4 *a, const uint4 *b, uint4 *y, unsigned n8)
{
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n8; i += gridDim.x * blockDim.x) {
        float fa[8], fb[8];
        unpack8(a[i], fa);
        unpack8(b[i], fb);
#pragma unroll
        for (int e = 0; e < 8; ++e) fa[e] += fb[e];
        y[i] = pack8(fa);
    }
}

// Output unit i of [N][H][W][CU] (H, W the output size) from input unit (n, yy / 2, xx / 2).
__global__ void k_up2_v(const uint4 *x, uint4 *y, unsigned N, unsigned H, unsigned W, unsigned CU)
{
    const unsigned total = N * H * W * CU;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const unsigned cu = i % CU, t = i / CU, xx = t % W, t2 = t / W, yy = t2 % H, n = t2 / H;
        y[i] = x[((n * (H / 2) + yy / 2) * (W / 2) + xx / 2) * CU + cu];
    }
}

// Input-gradient unit i of [N][H][W][CU] (H, W the input size): the sum of its four output units.
__global__ void k_up2_bwd_v(const uint4 *gy, uint4 *gx, unsigned N, unsigned H, unsigned W, unsigned CU)
{
    const unsigned total = N * H * W * CU;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const unsigned cu = i % CU, t = i / CU, x = t % W, t2 = t / W, yv = t2 % H, n = t2 / H;
        const size_t b = ((size_t)(n * 2 * H + 2 * yv) * (2 * W) + 2 * x) * CU + cu, row = (size_t)2 * W * CU;
        float s[8], f[8];
        unpack8(gy[b], s);
        unpack8(gy[b + CU], f);
#pragma unroll
        for (int e = 0; e < 8; ++e) s[e] += f[e];
        unpack8(gy[b + row], f);
#pragma unroll
        for (int e = 0; e < 8; ++e) s[e] += f[e];
        unpack8(gy[b + row + CU], f);
#pragma unroll
        for (int e = 0; e < 8; ++e) s[e] += f[e];
        gx[i] = pack8(s);
    }
}

// Output unit i of [N][H/2][W/2][CU] (H, W the input size): the mean of its four input units.
__global__ void k_pool2_v(const uint4 *x, uint4 *y, unsigned N, unsigned H, unsigned W, unsigned CU)
{
    const unsigned Ho = H / 2, Wo = W / 2, total = N * Ho * Wo * CU;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const unsigned cu = i % CU, t = i / CU, xo = t % Wo, t2 = t / Wo, yo = t2 % Ho, n = t2 / Ho;
        const size_t b = ((size_t)(n * H + 2 * yo) * W + 2 * xo) * CU + cu, row = (size_t)W * CU;
        float s[8], f[8];
        unpack8(x[b], s);
        unpack8(x[b + CU], f);
#pragma unroll
        for (int e = 0; e < 8; ++e) s[e] += f[e];
        unpack8(x[b + row], f);
#pragma unroll
        for (int e = 0; e < 8; ++e) s[e] += f[e];
        unpack8(x[b + row + CU], f);
#pragma unroll
        for (int e = 0; e < 8; ++e) s[e] = 0.25f * (s[e] + f[e]);
        y[i] = pack8(s);
    }
}

// Input-gradient unit i of [N][H][W][CU] (H, W the input size): a quarter of its pooled unit.
__global__ void k_pool2_bwd_v(const uint4 *gy, uint4 *gx, unsigned N, unsigned H, unsigned W, unsigned CU)
{
    const unsigned total = N * H * W * CU;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const unsigned cu = i % CU, t = i / CU, x = t % W, t2 = t / W, yv = t2 % H, n = t2 / H;
        float f[8];
        unpack8(gy[((size_t)(n * (H / 2) + yv / 2) * (W / 2) + x / 2) * CU + cu], f);
#pragma unroll
        for (int e = 0; e < 8; ++e) f[e] *= 0.25f;
        gx[i] = pack8(f);
    }
}

int grid_for(long long n) { return (int)((n + 255) / 256 < 152 * 16 ? (n + 255) / 256 : 152 * 16); }

// The 16-byte forms apply: C a multiple of 8, every pointer 16-byte aligned, units below 2^31.
bool vec8(int C, long long elems, const void *a, const void *b = nullptr, const void *c = nullptr)
{
    const auto al = [](const void *p) { return p == nullptr || ((uintptr_t)p & 15u) == 0; };
    return C % 8 == 0 && elems % 8 == 0 && elems / 8 < (1ll << 31) && al(a) && al(b) && al(c);
}

// gb[c] += sum over the P pixels of g[p][c]; with y, the ReLU backward of g first, in place (the
// 16-byte kernel needs C a multiple of 8 and aligned buffers; y without them is applied by the caller).
int bias_grad(const void *y, void *g, float *gb, long long P, int C, cudaStream_t s)
{
    if (vec8(C, P * C, g, y)) {
        const int CU = C / 8, threads = (256 / CU) * CU;
        const long long R = threads / CU;
        const int blocks = (int)((P + R - 1) / R < 152 * 4 ? (P + R - 1) / R : 152 * 4);
        if (y)
            k_bias_grad_v<true><<<blocks, threads, threads * 8 * sizeof(float), s>>>((const uint4 *)y, (uint4 *)g, gb,
                                                                                   (unsigned)P, CU);
        else
            k_bias_grad_v<false><<<blocks, threads, threads * 8 * sizeof(float), s>>>(nullptr, (uint4 *)g, gb,
                                                                                    (unsigned)P, CU);
        return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
    }
    const long long gx = (P + 7) / 8 < 1024 ? (P + 7) / 8 : 1024;
    dim3 grid((unsigned)gx, (unsigned)((C + 31) / 32));
    k_bias_grad<<<grid, 256, 0, s>>>((const __nv_bfloat16 *)g, gb, P, C);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

template <int MODE>
int run_conv(ConvArgs a, cudaStream_t s)
{
    dim3 grid((a.M + BM - 1) / BM, (a.Ncols + BN - 1) / BN, 1);
    if (MODE == WGRAD) {
        const int splits = 152 * 2 / max(1, (int)(grid.x * grid.y)) + 1;
        a.k_chunk = ((a.K + splits - 1) / splits + BK - 1) / BK * BK;
        grid.z = (a.K + a.k_chunk - 1) / a.k_chunk;
    }
    k_conv<MODE><<<grid, THREADS, 0, s>>>(a);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

}  // namespace

extern "C" {

int plbm_nn_conv_fwd(const void *x, const void *w, const float *bias, void *y, int N, int H, int W, int Cin,
                     int Cout, int relu, void *stream)
{
    if (plbm_nn_tc_supported(H, W, Cin, Cout))
        return plbm_nn_tc_conv(x, w, bias, y, N, H, W, Cin, Cout, relu, (cudaStream_t)stream);
    if (plbm_nn_tc_small_supported(H, W, Cin, Cout))
        return plbm_nn_tc_small_conv(x, w, bias, y, N, H, W, Cin, Cout, relu, (cudaStream_t)stream);
    ConvArgs a{};
    a.x = (const __nv_bfloat16 *)x; a.w = (const __nv_bfloat16 *)w; a.bias = bias; a.y = (__nv_bfloat16 *)y;
    a.N = N; a.H = H; a.W = W; a.Cin = Cin; a.Cout = Cout; a.relu = relu;
    a.M = N * H * W; a.Ncols = Cout; a.K = 9 * Cin;
    return run_conv<FWD>(a, (cudaStream_t)stream);
}

int plbm_nn_flip_layers(const void *w, void *wt, const int *segs, int layers, int max_elems, void *stream)
{
    if (layers <= 0 || layers > 65535 || max_elems <= 0 || !segs) return PLBM_ERR_ARGUMENT;
    const dim3 grid((unsigned)((max_elems + 255) / 256 < 64 ? (max_elems + 255) / 256 : 64), (unsigned)layers);
    k_flip_layers<<<grid, 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)w, (__nv_bfloat16 *)wt, segs);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

int plbm_nn_conv_dgrad_pre(const void *g, const void *w, const void *wt, void *gx, int N, int H, int W, int Cin,
                           int Cout, void *stream)
{
    const bool tma = plbm_nn_tc_supported(H, W, Cout, Cin);
    if (tma) return plbm_nn_tc_conv(g, wt, nullptr, gx, N, H, W, Cout, Cin, 0, (cudaStream_t)stream);
    if (plbm_nn_tc_small_supported(H, W, Cout, Cin))
        return plbm_nn_tc_small_conv(g, wt, nullptr, gx, N, H, W, Cout, Cin, 0, (cudaStream_t)stream);
    return plbm_nn_conv_dgrad(g, w, gx, N, H, W, Cin, Cout, stream);
}

int plbm_nn_conv_dgrad(const void *g, const void *w, void *gx, int N, int H, int W, int Cin, int Cout, void *stream)
{
    // gx = conv3x3(g, W') with W'[ci][tap][co] = W[co][8 - tap][ci]: a forward kernel on the
    // tensor cores (the TMA one, or for a narrow gradient the one with thread-written tiles), with
    // the re-laid-out weights in a buffer kept for the process
    const bool tma = plbm_nn_tc_supported(H, W, Cout, Cin);
    if (tma || plbm_nn_tc_small_supported(H, W, Cout, Cin)) {
        // a buffer that grows is replaced, not freed: a CUDA graph captured earlier may still
        // launch with the old pointer
        static std::mutex mu;
        static void *wt = nullptr;
        static size_t cap = 0;
        const size_t need = (size_t)Cin * 9 * Cout * 2;
        std::lock_guard<std::mutex> lock(mu);
        if (need > cap) {
            void *p = nullptr;
            if (cudaMalloc(&p, need) != cudaSuccess) return PLBM_ERR_CUDA;
            wt = p;
            cap = need;
        }
        const int rc = plbm_nn_tc_flip(w, wt, Cin, Cout, (cudaStream_t)stream);
        if (rc != PLBM_OK) return rc;
        return tma ? plbm_nn_tc_conv(g, wt, nullptr, gx, N, H, W, Cout, Cin, 0, (cudaStream_t)stream)
                   : plbm_nn_tc_small_conv(g, wt, nullptr, gx, N, H, W, Cout, Cin, 0, (cudaStream_t)stream);
    }
    ConvArgs a{};
    a.g = (const __nv_bfloat16 *)g; a.w = (const __nv_bfloat16 *)w; a.y = (__nv_bfloat16 *)gx;
    a.N = N; a.H = H; a.W = W; a.Cin = Cin; a.Cout = Cout;
    a.M = N * H * W; a.Ncols = Cin; a.K = 9 * Cout;
    return run_conv<DGRAD>(a, (cudaStream_t)stream);
}

int plbm_nn_conv_wgrad(const void *x, const void *g, float *gw, float *gb, int N, int H, int W, int Cin, int Cout,
                       void *stream)
{
    int rc;
    if (plbm_nn_tc_wgrad_supported(H, W, Cin, Cout)) {
        int bias_done = 0;
        rc = plbm_nn_tc_wgrad(x, g, gw, gb, N, H, W, Cin, Cout, &bias_done, (cudaStream_t)stream);
        if (bias_done) gb = nullptr;   // the bias gradient came with the weight gradient
    } else if (plbm_nn_tc_small_wgrad_supported(H, W, Cin, Cout)) {
        rc = plbm_nn_tc_small_wgrad(x, g, gw, N, H, W, Cin, Cout, (cudaStream_t)stream);
    } else {
        ConvArgs a{};
        a.x = (const __nv_bfloat16 *)x; a.g = (const __nv_bfloat16 *)g; a.gw = gw;
        a.N = N; a.H = H; a.W = W; a.Cin = Cin; a.Cout = Cout;
        a.M = Cout; a.Ncols = 9 * Cin; a.K = N * H * W;
        rc = run_conv<WGRAD>(a, (cudaStream_t)stream);
    }
    // without y the bias kernel only reads g
    if (rc == PLBM_OK && gb)
        rc = bias_grad(nullptr, const_cast<void *>(g), gb, (long long)N * H * W, Cout, (cudaStream_t)stream);
    return rc;
}

int plbm_nn_relu_bwd_bias(const void *y, void *g, float *gb, long long P, int C, void *stream)
{
    if (P <= 0 || C <= 0 || !gb) return PLBM_ERR_ARGUMENT;
    if (!vec8(C, P * C, y, g)) {
        const int rc = plbm_nn_relu_bwd(y, g, P * C, stream);
        return rc == PLBM_OK ? bias_grad(nullptr, g, gb, P, C, (cudaStream_t)stream) : rc;
    }
    return bias_grad(y, g, gb, P, C, (cudaStream_t)stream);
}

int plbm_nn_relu_bwd(const void *y, void *g, long long n, void *stream)
{
    if (vec8(8, n, y, g)) {
        k_relu_bwd_v<<<grid_for(n / 8), 256, 0, (cudaStream_t)stream>>>((const uint4 *)y, (uint4 *)g, (unsigned)(n / 8));
        return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
    }
    k_relu_bwd<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)y, (__nv_bfloat16 *)g, n);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

int plbm_nn_pool2(const void *x, void *y, int N, int H, int W, int C, void *stream)
{
    if (vec8(C, (long long)N * H * W * C, x, y)) {
        k_pool2_v<<<grid_for((long long)N * H * W * C / 32), 256, 0, (cudaStream_t)stream>>>(
            (const uint4 *)x, (uint4 *)y, N, H, W, C / 8);
        return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
    }
    k_pool2<<<grid_for((long long)N * H * W * C / 4), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)x,
                                                                                       (__nv_bfloat16 *)y, N, H, W, C);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

int plbm_nn_pool2_bwd(const void *gy, void *gx, int N, int H, int W, int C, void *stream)
{
    if (vec8(C, (long long)N * H * W * C, gy, gx)) {
        k_pool2_bwd_v<<<grid_for((long long)N * H * W * C / 8), 256, 0, (cudaStream_t)stream>>>(
            (const uint4 *)gy, (uint4 *)gx, N, H, W, C / 8);
        return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
    }
    k_pool2_bwd<<<grid_for((long long)N * H * W * C), 256, 0, (cudaStream_t)stream>>>(
        (const __nv_bfloat16 *)gy, (__nv_bfloat16 *)gx, N, H, W, C);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

int plbm_nn_up2(const void *x, void *y, int N, int H, int W, int C, void *stream)
{
    if (vec8(C, (long long)N * H * W * C, x, y)) {
        k_up2_v<<<grid_for((long long)N * H * W * C / 8), 256, 0, (cudaStream_t)stream>>>(
            (const uint4 *)x, (uint4 *)y, N, H, W, C / 8);
        return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
    }
    k_up2<<<grid_for((long long)N * H * W * C), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)x,
                                                                                 (__nv_bfloat16 *)y, N, H, W, C);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

int plbm_nn_up2_bwd(const void *gy, void *gx, int N, int H, int W, int C, void *stream)
{
    if (vec8(C, (long long)N * H * W * C * 4, gy, gx)) {
        k_up2_bwd_v<<<grid_for((long long)N * H * W * C / 8), 256, 0, (cudaStream_t)stream>>>(
            (const uint4 *)gy, (uint4 *)gx, N, H, W, C / 8);
        return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
    }
    k_up2_bwd<<<grid_for((long long)N * H * W * C), 256, 0, (cudaStream_t)stream>>>(
        (const __nv_bfloat16 *)gy, (__nv_bfloat16 *)gx, N, H, W, C);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

int plbm_nn_add(const void *a, const void *b, void *y, long long n, void *stream)
{
    if (vec8(8, n, a, b, y)) {
        k_add_v<<<grid_for(n / 8), 256, 0, (cudaStream_t)stream>>>((const uint4 *)a, (const uint4 *)b, (uint4 *)y,
                                                                  (unsigned)(n / 8));
        return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
    }
    k_add<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)a, (const __nv_bfloat16 *)b,
                                                         (__nv_bfloat16 *)y, n);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

int plbm_nn_mse(const void *pred, const float *target, const int8_t *mask, void *grad, float *loss, long long P, int C,
                float inv_count, void *stream)
{
    k_mse<<<grid_for(P * C), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)pred, target, mask,
                                                             (__nv_bfloat16 *)grad, loss, P, C, inv_count);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

int plbm_nn_adam(float *w, const float *g, float *m, float *v, void *wb, long long n, float lr, float b1, float b2,
                 float eps, int t, void *stream)
{
    const float c1 = 1.f / (1.f - powf(b1, (float)t)), c2 = 1.f / (1.f - powf(b2, (float)t));
    k_adam<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, (__nv_bfloat16 *)wb, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

int plbm_nn_adam_dev(float *w, const float *g, float *m, float *v, void *wb, long long n, const float *lr, float b1,
                     float b2, float eps, int *state, void *stream)
{
    if (n <= 0 || !lr || !state) return PLBM_ERR_ARGUMENT;
    k_adam_dev<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, (__nv_bfloat16 *)wb, n, lr, b1, b2, eps,
                                                             state);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

int plbm_nn_assemble(const int8_t *mask, const float *features, void *y, int N, int H, int W, int C, void *stream)
{
    if (N <= 0 || H <= 0 || W <= 0 || C < 4) return PLBM_ERR_ARGUMENT;
    k_assemble<<<grid_for((long long)N * H * W), 256, 0, (cudaStream_t)stream>>>(mask, features, (__nv_bfloat16 *)y,
                                                                                 N, H, W, C);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

}  // extern "C"
