// plbm_nn_tc.cu — the warm-start operator's 3x3 convolution on the 5th-generation tensor cores.
//
// Implicit GEMM: out[pixel, co] = sum over the 9 taps and Cin of x[pixel + tap, ci] * W[co, tap, ci].
// A CTA owns 128 output pixels (a BW x BH block of one image, BW = min(W, 128)) and all Cout (padded
// to a multiple of 16).  The K loop walks (tap, 32-channel block); for each step a TMA tensor load
// brings the 128 shifted input pixels x 32 channels (zero-filled outside the image) and a tensor
// load brings Npad x 32 weights, both as 64-byte rows with the 64-byte swizzle, i.e. the canonical
// K-major layout of the tensor-core shared-memory descriptors.  One thread issues
// tcgen05.mma (kind::f16, BF16 x BF16 -> FP32) into a TMEM accumulator of 128 lanes x Npad
// columns; the stage is released by tcgen05.commit on its mbarrier.  Four warps then read the
// accumulator with tcgen05.ld (warp w: lanes 32w..32w+31), add the bias, apply ReLU and store BF16
// NHWC.  The input gradient of a convolution is the same computation on the gradient with the
// weights transposed in channels and flipped in taps (k_flip_weights).
//
// Every wait is bounded (about 1 s): on expiry the thread records an error in g_tc_error, stops
// its role, waits (bounded) for its own copies in flight, the CTA frees its TMEM and returns.
#include "../../include/plbm_c.h"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <mutex>

namespace {

constexpr int TC_BM = 128;          // output pixels per CTA (TMEM lanes)
constexpr int TC_KB = 32;           // channels per K block (64-byte rows)
constexpr int TC_STAGES = 4;
constexpr int TC_A_BYTES = TC_BM * TC_KB * 2;        // 8 KB
constexpr int TC_B_MAX = 128 * TC_KB * 2;            // 8 KB at Npad = 128
constexpr int TC_SMEM = TC_STAGES * (TC_A_BYTES + TC_B_MAX) + 1024 /* alignment */ + 256 /* barriers */;   // largest
constexpr long long TC_WAIT_CYCLES = 2000000000ll;   // ~1 s at the maximum SM clock

__device__ int g_tc_error;

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned n)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(n) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(unsigned bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity)
{
    const long long t0 = clock64();
    while (!mbar_try(bar, parity))
        if (clock64() - t0 > TC_WAIT_CYCLES) return false;
    return true;
}

__device__ __forceinline__ void tma_load_4d(unsigned dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            unsigned bar)
{
    asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
                 ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
                 : "memory");
}
__device__ __forceinline__ void tma_load_3d(unsigned dst, const CUtensorMap *map, int c0, int c1, int c2, unsigned bar)
{
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
                 ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
                 : "memory");
}

// Shared-memory matrix descriptor: K-major operand in 64-byte-swizzled rows; 8-row groups 512 B
// apart (stride byte offset), leading byte offset unused for swizzled K-major (set to 1).
__device__ __forceinline__ uint64_t smem_desc_sw64(unsigned addr)
{
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(512 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)4 << 61);
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both K-major, N x M = npad x 128.
__device__ __forceinline__ unsigned instr_desc(int npad)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(npad >> 3) << 17) | ((unsigned)(TC_BM >> 4) << 24);
}

__device__ __forceinline__ void umma(unsigned tmem, uint64_t a, uint64_t b, unsigned idesc, bool acc)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                 ::"r"(tmem), "l"(a), "l"(b), "r"(idesc), "r"((unsigned)acc)
                 : "memory");
}
__device__ __forceinline__ void umma_commit(unsigned bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

struct TcArgs {
    __nv_bfloat16 *y;
    const float *bias;      // may be null
    int N, H, W, Cin, Cout, npad, relu;
    int BW, BH, tiles_x, tiles_y;
    int stage_bytes;        // A tile + the B tile rounded up to 1024 B
    int *err;
};

__global__ void __launch_bounds__(128, 4)
k_conv_tc(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap wmap, TcArgs a)
{
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    // stages aligned to 1024 B (the swizzle pattern repeats every 512 B)
    unsigned char *smem = tc_smem_raw + ((1024 - (smem_u32(tc_smem_raw) & 1023)) & 1023);
    unsigned long long *bars = reinterpret_cast<unsigned long long *>(smem + TC_STAGES * a.stage_bytes);
    unsigned long long *full = bars, *empty = bars + TC_STAGES, *done = bars + 2 * TC_STAGES;
    unsigned *tmem_slot = reinterpret_cast<unsigned *>(bars + 2 * TC_STAGES + 1);
    int *counts = reinterpret_cast<int *>(tmem_slot + 1);   // [0] issued, [1] consumed, [2] failed

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned ncols = a.npad <= 32 ? 32u : (a.npad <= 64 ? 64u : 128u);
    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; ++s) { mbar_init(smem_u32(&full[s]), 1); mbar_init(smem_u32(&empty[s]), 1); }
        mbar_init(smem_u32(done), 1);
        counts[0] = counts[1] = counts[2] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(ncols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = *tmem_slot;

    // tile -> image n, block origin (x0, y0)
    const int tile = blockIdx.x;
    const int per_img = a.tiles_x * a.tiles_y;
    const int n = tile / per_img, t2 = tile % per_img;
    const int y0 = (t2 / a.tiles_x) * a.BH, x0 = (t2 % a.tiles_x) * a.BW;
    const int kblocks = a.Cin / TC_KB, iters = 9 * kblocks;
    const unsigned bbytes = (unsigned)a.npad * TC_KB * 2;

    if (warp == 0 && lane == 0) {              // producer: TMA loads
        for (int it = 0; it < iters; ++it) {
            const int s = it % TC_STAGES;
            if (it >= TC_STAGES && !mbar_wait(smem_u32(&empty[s]), (unsigned)((it / TC_STAGES - 1) & 1))) {
                counts[2] = 1;
                break;
            }
            const int tap = it / kblocks, kb = it % kblocks;
            const int dy = tap / 3 - 1, dx = tap % 3 - 1;
            unsigned char *st = smem + s * a.stage_bytes;
            const unsigned bar = smem_u32(&full[s]);
            mbar_expect_tx(bar, (unsigned)TC_A_BYTES + bbytes);
            tma_load_4d(smem_u32(st), &xmap, kb * TC_KB, x0 + dx, y0 + dy, n, bar);
            tma_load_3d(smem_u32(st + TC_A_BYTES), &wmap, kb * TC_KB, tap, 0, bar);
            counts[0] = it + 1;
        }
    } else if (warp == 1 && lane == 0) {       // MMA issuer
        const unsigned idesc = instr_desc(a.npad);
        int it = 0;
        for (; it < iters; ++it) {
            const int s = it % TC_STAGES;
            if (!mbar_wait(smem_u32(&full[s]), (unsigned)((it / TC_STAGES) & 1))) {
                counts[2] = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const unsigned abase = smem_u32(smem + s * a.stage_bytes), bbase = abase + TC_A_BYTES;
#pragma unroll
            for (int k = 0; k < TC_KB / 16; ++k)   // K = 16 per MMA: +32 B along the swizzled row
                umma(tmem, smem_desc_sw64(abase + 32 * k), smem_desc_sw64(bbase + 32 * k), idesc, it > 0 || k > 0);
            umma_commit(smem_u32(&empty[s]));
            counts[1] = it + 1;
        }
        umma_commit(smem_u32(done));               // arrives when every issued MMA has completed
    }
    // epilogue: all four warps, once every role has finished
    if (!mbar_wait(smem_u32(done), 0)) counts[2] = 1;
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int row = warp * 32 + lane;
    const int px = x0 + row % a.BW, py = y0 + row / a.BW;
    const bool valid = *((volatile int *)&counts[2]) == 0;
    for (int c0 = 0; c0 < a.npad; c0 += 16) {
        unsigned v[16];
        const unsigned taddr = tmem + ((unsigned)(warp * 32) << 16) + (unsigned)c0;
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                     : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                       "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                     : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (!valid || py >= a.H || px >= a.W) continue;
        __nv_bfloat16 *out = a.y + (((size_t)n * a.H + py) * a.W + px) * a.Cout;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int co = c0 + j;
            if (co < a.Cout) {
                float f = __uint_as_float(v[j]) + (a.bias ? a.bias[co] : 0.f);
                if (a.relu) f = fmaxf(f, 0.f);
                out[co] = __float2bfloat16_rn(f);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0 && !valid) {
        atomicExch(a.err, 1);
        // after a failed wait: the MMAs issued (their completion barrier) and the copies still in
        // flight (their stages' full barriers), each bounded, before the TMEM is released
        mbar_wait(smem_u32(done), 0);
        for (int it = counts[1]; it < counts[0]; ++it)
            mbar_wait(smem_u32(&full[it % TC_STAGES]), (unsigned)((it / TC_STAGES) & 1));
    }
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
    }
}

// ---- weight gradient ------------------------------------------------------------------------
// dW[co][tap][ci] += sum over pixels p of g[p][co] * x[p + offset(tap)][ci]: a GEMM with M = Cout,
// N = Cin per tap and K = the pixels.  Both operands arrive as TMA tiles of 128 pixels x 32
// channels (64-byte rows, 64-byte swizzle), exactly the tiles of the forward kernel: a row is one
// pixel, i.e. one K index, holding 32 consecutive M (or N) elements, so both are fed to tcgen05.mma
// MN-major ("transposed" in the instruction descriptor).  In that layout a swizzle atom is 8 K-rows
// of 32 MN elements; the stride byte offset steps 8 K-rows (512 B) and the leading byte offset
// steps 32 MN elements (the next 32-channel tile, WG_CHUNK bytes on).  M is Cout padded to 128
// (TMA fills the channels past Cout with zeros); each of the CTA's taps accumulates N = Cin TMEM
// columns.  A CTA walks (pixel tile, tap) pairs of its share of the pixels (split K, one CTA per
// SM) and adds its partial sums to dW with FP32 atomics.
constexpr int WG_M = 128;                          // TMEM lanes: Cout padded
constexpr int WG_CHUNK = TC_BM * TC_KB * 2;        // one 128-pixel x 32-channel tile, 8 KB
constexpr int WG_A_BYTES = (WG_M / TC_KB) * WG_CHUNK;   // 32 KB
constexpr int WG_SLACK = 16384;                    // keeps any reading of the descriptors inside the allocation

struct WgArgs {
    float *gw;
    int N, H, W, Cin, Cout;
    int BW, BH, tiles_x, tiles_y;
    int ntaps;              // taps per CTA (3 or 9); blockIdx.y selects the group
    int tiles_per_cta, total_tiles;
    int b_bytes, stage_bytes, stages;
    int *err;
};

// MN-major operand in 64-byte-swizzled rows: leading byte offset = next 32-element MN tile,
// stride byte offset = next group of 8 K-rows (512 B).
__device__ __forceinline__ uint64_t smem_desc_mn_sw64(unsigned addr, unsigned lbo_bytes)
{
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo_bytes >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)(512 >> 4) << 32) | ((uint64_t)1 << 46) | ((uint64_t)4 << 61);
}

// kind::f16, FP32 accumulator, BF16 A and B, both MN-major, M = 128, N = n.
__device__ __forceinline__ unsigned instr_desc_mn(int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) | ((unsigned)(n >> 3) << 17) |
           ((unsigned)(WG_M >> 4) << 24);
}

__global__ void __launch_bounds__(128, 1)
k_wgrad_tc(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap gmap, WgArgs a)
{
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    unsigned char *smem = tc_smem_raw + ((1024 - (smem_u32(tc_smem_raw) & 1023)) & 1023);
    unsigned long long *bars = reinterpret_cast<unsigned long long *>(smem + a.stages * a.stage_bytes + WG_SLACK);
    unsigned long long *full = bars, *empty = bars + a.stages, *done = bars + 2 * a.stages;
    unsigned *tmem_slot = reinterpret_cast<unsigned *>(bars + 2 * a.stages + 1);
    int *counts = reinterpret_cast<int *>(tmem_slot + 1);   // [0] issued, [1] consumed, [2] failed

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cols = a.ntaps * a.Cin;
    const unsigned ncols = cols <= 32 ? 32u : cols <= 64 ? 64u : cols <= 128 ? 128u : cols <= 256 ? 256u : 512u;
    if (threadIdx.x == 0) {
        for (int s = 0; s < a.stages; ++s) { mbar_init(smem_u32(&full[s]), 1); mbar_init(smem_u32(&empty[s]), 1); }
        mbar_init(smem_u32(done), 1);
        counts[0] = counts[1] = counts[2] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(ncols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = *tmem_slot;

    const int tap0 = blockIdx.y * a.ntaps;
    const int first = blockIdx.x * a.tiles_per_cta;
    const int ntiles = max(0, min(a.tiles_per_cta, a.total_tiles - first));
    const int iters = ntiles * a.ntaps;
    const int per_img = a.tiles_x * a.tiles_y;
    const int kbx = a.Cin / TC_KB;

    if (warp == 0 && lane == 0) {              // producer: TMA loads of the g tile and the shifted x tile
        for (int it = 0; it < iters; ++it) {
            const int s = it % a.stages;
            if (it >= a.stages && !mbar_wait(smem_u32(&empty[s]), (unsigned)((it / a.stages - 1) & 1))) {
                counts[2] = 1;
                break;
            }
            const int tile = first + it / a.ntaps, tap = tap0 + it % a.ntaps;
            const int n = tile / per_img, t2 = tile % per_img;
            const int y0 = (t2 / a.tiles_x) * a.BH, x0 = (t2 % a.tiles_x) * a.BW;
            const int dy = tap / 3 - 1, dx = tap % 3 - 1;
            unsigned char *st = smem + s * a.stage_bytes;
            const unsigned bar = smem_u32(&full[s]);
            mbar_expect_tx(bar, (unsigned)WG_A_BYTES + (unsigned)a.b_bytes);
            for (int c = 0; c < WG_M / TC_KB; ++c)
                tma_load_4d(smem_u32(st + c * WG_CHUNK), &gmap, c * TC_KB, x0, y0, n, bar);
            for (int c = 0; c < kbx; ++c)
                tma_load_4d(smem_u32(st + WG_A_BYTES + c * WG_CHUNK), &xmap, c * TC_KB, x0 + dx, y0 + dy, n, bar);
            counts[0] = it + 1;
        }
    } else if (warp == 1 && lane == 0) {       // MMA issuer
        const unsigned idesc = instr_desc_mn(a.Cin);
        int it = 0;
        for (; it < iters; ++it) {
            const int s = it % a.stages;
            if (!mbar_wait(smem_u32(&full[s]), (unsigned)((it / a.stages) & 1))) {
                counts[2] = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const unsigned abase = smem_u32(smem + s * a.stage_bytes), bbase = abase + WG_A_BYTES;
            const unsigned dcol = tmem + (unsigned)((it % a.ntaps) * a.Cin);
            const bool first_tile = it < a.ntaps;
#pragma unroll
            for (int k = 0; k < TC_BM / 16; ++k)   // K = 16 pixels per MMA: two 8-row groups, 1 KB on
                umma(dcol, smem_desc_mn_sw64(abase + 1024 * k, WG_CHUNK), smem_desc_mn_sw64(bbase + 1024 * k, WG_CHUNK),
                     idesc, !(first_tile && k == 0));
            umma_commit(smem_u32(&empty[s]));
            counts[1] = it + 1;
        }
        umma_commit(smem_u32(done));
    }
    if (!mbar_wait(smem_u32(done), 0)) counts[2] = 1;
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool valid = *((volatile int *)&counts[2]) == 0;
    const int co = warp * 32 + lane;
    if (iters > 0) {
        for (int c0 = 0; c0 < cols; c0 += 16) {
            unsigned v[16];
            const unsigned taddr = tmem + ((unsigned)(warp * 32) << 16) + (unsigned)c0;
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                         : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                           "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                         : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (!valid || co >= a.Cout) continue;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int col = c0 + j, t = col / a.Cin, ci = col % a.Cin;
                atomicAdd(&a.gw[(size_t)co * 9 * a.Cin + (size_t)(tap0 + t) * a.Cin + ci], __uint_as_float(v[j]));
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0 && !valid) {
        atomicExch(a.err, 1);
        mbar_wait(smem_u32(done), 0);
        for (int it = counts[1]; it < counts[0]; ++it)
            mbar_wait(smem_u32(&full[it % a.stages]), (unsigned)((it / a.stages) & 1));
    }
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
    }
}

// Wt[ci][tap][co] = W[co][8 - tap][ci]: the weights of the input-gradient convolution.
__global__ void k_flip_weights(const __nv_bfloat16 *w, __nv_bfloat16 *wt, int Cin, int Cout)
{
    const int total = Cout * 9 * Cin;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int co = i / (9 * Cin), r = i % (9 * Cin), tap = r / Cin, ci = r % Cin;
        wt[((size_t)ci * 9 + (8 - tap)) * Cout + co] = w[i];
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

int *error_flag()
{
    static int *p = nullptr;
    static std::once_flag once;
    std::call_once(once, [] { cudaGetSymbolAddress((void **)&p, g_tc_error); });
    return p;
}

}  // namespace

// The tensor-core path covers Cin a multiple of 32, Cout <= 128, and images tiled exactly by
// 128-pixel blocks (W a multiple of 128, or a power of two below it with H a multiple of 128 / W).
bool plbm_nn_tc_supported(int H, int W, int Cin, int Cout)
{
    if (Cin % TC_KB != 0 || Cin > 4096 || Cout < 1 || Cout > 128) return false;
    if (W % TC_BM == 0) return true;
    if (TC_BM % W != 0) return false;
    return H % (TC_BM / W) == 0;
}

// y = act(conv3x3(x, w) + bias) on the tensor cores; x, y NHWC BF16; w [Cout][9][Cin] BF16.
int plbm_nn_tc_conv(const void *x, const void *w, const float *bias, void *y, int N, int H, int W, int Cin, int Cout,
                    int relu, cudaStream_t s)
{
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    int *err = error_flag();
    if (!enc || !err) return PLBM_ERR_CUDA;
    static bool attr = false;
    static std::mutex mu;
    {
        std::lock_guard<std::mutex> g(mu);
        if (!attr) {
            if (cudaFuncSetAttribute(k_conv_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM) != cudaSuccess)
                return PLBM_ERR_CUDA;
            attr = true;
        }
    }
    const int BW = W >= TC_BM ? TC_BM : W, BH = TC_BM / BW;
    const int npad = (Cout + 15) / 16 * 16;
    CUtensorMap xmap, wmap;
    {
        const cuuint64_t dims[4] = { (cuuint64_t)Cin, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N };
        const cuuint64_t strides[3] = { (cuuint64_t)Cin * 2, (cuuint64_t)W * Cin * 2, (cuuint64_t)H * W * Cin * 2 };
        const cuuint32_t box[4] = { TC_KB, (cuuint32_t)BW, (cuuint32_t)BH, 1 };
        const cuuint32_t es[4] = { 1, 1, 1, 1 };
        if (enc(&xmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(x), dims, strides, box, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return PLBM_ERR_ARGUMENT;
    }
    {
        const cuuint64_t dims[3] = { (cuuint64_t)Cin, 9, (cuuint64_t)Cout };
        const cuuint64_t strides[2] = { (cuuint64_t)Cin * 2, (cuuint64_t)9 * Cin * 2 };
        const cuuint32_t box[3] = { TC_KB, 1, (cuuint32_t)npad };
        const cuuint32_t es[3] = { 1, 1, 1 };
        if (enc(&wmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(w), dims, strides, box, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return PLBM_ERR_ARGUMENT;
    }
    // stages sized by the padded output channels, so narrow layers fit more CTAs per SM
    const int stage = TC_A_BYTES + (npad * TC_KB * 2 + 1023) / 1024 * 1024;
    TcArgs a{ (__nv_bfloat16 *)y, bias, N, H, W, Cin, Cout, npad, relu, BW, BH, W / BW, H / BH, stage, err };
    const int tiles = N * a.tiles_x * a.tiles_y;
    k_conv_tc<<<tiles, 128, TC_STAGES * stage + 1024 + 256, s>>>(xmap, wmap, a);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

// The weight gradient runs on the tensor cores for Cin and Cout multiples of 32 up to 128 and the
// image tilings of the forward kernel.
bool plbm_nn_tc_wgrad_supported(int H, int W, int Cin, int Cout)
{
    if (Cin % TC_KB != 0 || Cout % TC_KB != 0 || Cin > 128 || Cout > WG_M || Cin < TC_KB) return false;
    return plbm_nn_tc_supported(H, W, Cin, Cout);
}

// gw[co][tap][ci] += sum_p g[p][co] x[p + tap][ci] on the tensor cores (x, g NHWC BF16, gw FP32).
int plbm_nn_tc_wgrad(const void *x, const void *g, float *gw, int N, int H, int W, int Cin, int Cout, cudaStream_t s)
{
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    int *err = error_flag();
    if (!enc || !err) return PLBM_ERR_CUDA;
    const int BW = W >= TC_BM ? TC_BM : W, BH = TC_BM / BW;
    const int ntaps = 9 * Cin <= 512 ? 9 : 3;
    const int b_bytes = (Cin / TC_KB) * WG_CHUNK;
    const int stage = WG_A_BYTES + b_bytes;
    const int stages = (200 * 1024) / stage < 4 ? (200 * 1024) / stage : 4;
    const int smem = stages * stage + WG_SLACK + 1024 + 256;
    static int attr_bytes = 0;
    static std::mutex mu;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (smem > attr_bytes) {
            if (cudaFuncSetAttribute(k_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
                return PLBM_ERR_CUDA;
            attr_bytes = smem;
        }
    }
    CUtensorMap xmap, gmap;
    const cuuint32_t es[4] = { 1, 1, 1, 1 };
    for (int which = 0; which < 2; ++which) {
        const int C = which == 0 ? Cin : Cout;
        const cuuint64_t dims[4] = { (cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N };
        const cuuint64_t strides[3] = { (cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2 };
        const cuuint32_t box[4] = { TC_KB, (cuuint32_t)BW, (cuuint32_t)BH, 1 };
        if (enc(which == 0 ? &xmap : &gmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(which == 0 ? x : g),
                dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return PLBM_ERR_ARGUMENT;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    const int groups = 9 / ntaps;
    const int total = N * (W / BW) * (H / BH);
    const int chunks = (sms + groups - 1) / groups;
    const int per = (total + chunks - 1) / chunks;
    WgArgs a{ gw, N, H, W, Cin, Cout, BW, BH, W / BW, H / BH, ntaps, per, total, b_bytes, stage, stages, err };
    k_wgrad_tc<<<dim3((total + per - 1) / per, groups), 128, smem, s>>>(xmap, gmap, a);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

int plbm_nn_tc_flip(const void *w, void *wt, int Cin, int Cout, cudaStream_t s)
{
    const int total = Cout * 9 * Cin;
    k_flip_weights<<<(total + 255) / 256 < 1024 ? (total + 255) / 256 : 1024, 256, 0, s>>>(
        (const __nv_bfloat16 *)w, (__nv_bfloat16 *)wt, Cin, Cout);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

extern "C" int plbm_nn_conv_on_tensor_cores(int H, int W, int Cin, int Cout)
{
    return plbm_nn_tc_supported(H, W, Cin, Cout) ? 1 : 0;
}

extern "C" int plbm_nn_status(int *failed)
{
    int *err = error_flag();
    if (!err) return PLBM_ERR_CUDA;
    int v = 0;
    if (cudaMemcpy(&v, err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return PLBM_ERR_CUDA;
    if (failed) *failed = v;
    if (v) {
        const int zero = 0;
        cudaMemcpy(err, &zero, sizeof(int), cudaMemcpyHostToDevice);
    }
    return PLBM_OK;
}
