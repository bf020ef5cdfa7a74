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
#include <cstring>
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

// The bias of a CTA's output channels in shared memory (zero past Cout and without a bias), read by
// every epilogue thread: npad <= 128 floats.
__device__ __forceinline__ void stage_bias(float *sb, const float *bias, int Cout, int npad)
{
    for (int i = threadIdx.x; i < npad; i += blockDim.x) sb[i] = bias && i < Cout ? bias[i] : 0.f;
}

// Epilogue of one pixel: accumulator columns c0 .. c0 + 15 (FP32 bit patterns) plus the bias (sb,
// shared memory), ReLU, rounded to BF16 and stored to out[c0 ..] for the channels below C; with C
// a multiple of 8, as 16-byte stores of eight channels (a pixel row is 16-byte aligned then).
__device__ __forceinline__ void store_row16(__nv_bfloat16 *out, int c0, int C, const unsigned v[16], const float *sb,
                                            int relu)
{
    float f[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        f[j] = __uint_as_float(v[j]) + sb[c0 + j];
        if (relu) f[j] = fmaxf(f[j], 0.f);
    }
    if (C % 8 == 0) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (c0 + 8 * h >= C) break;
            uint32_t q[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                __nv_bfloat162 b2 = __floats2bfloat162_rn(f[8 * h + 2 * e], f[8 * h + 2 * e + 1]);
                q[e] = *reinterpret_cast<uint32_t *>(&b2);
            }
            *reinterpret_cast<uint4 *>(out + c0 + 8 * h) = make_uint4(q[0], q[1], q[2], q[3]);
        }
    } else {
#pragma unroll
        for (int j = 0; j < 16; ++j)
            if (c0 + j < C) out[c0 + j] = __float2bfloat16_rn(f[j]);
    }
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
    __shared__ float s_bias[128];
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
    stage_bias(s_bias, a.bias, a.Cout, a.npad);
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
        store_row16(a.y + (((size_t)n * a.H + py) * a.W + px) * a.Cout, c0, a.Cout, v, s_bias, a.relu);
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
// dW[co][tap][ci] += sum over pixels p of g[p][co] * x[p + offset(tap)][ci], computed as its
// transpose: a GEMM with M = the (tap, ci) rows, N = Cout and K = the pixels.  A stage holds, for
// one 128-pixel tile, the shifted input tiles of TG taps (TG * Cin / 32 TMA tiles of 128 pixels x 32
// channels, 64-byte rows with the 64-byte swizzle, exactly the tiles of the forward kernel) and the
// tile's output gradient (Cout / 32 such tiles, or for Cout < 32 written by two warps).  A row of
// either is one pixel, i.e. one K index, holding 32 consecutive M (or N) elements, so both are
// fed to tcgen05.mma MN-major ("transposed" in the instruction descriptor): a swizzle atom is 8
// K-rows of 32 MN elements, the stride byte offset steps 8 K-rows (512 B) and the leading byte
// offset the next 32-element tile (WG_CHUNK bytes on).  The stage's input tiles are covered by M
// tiles of four (128 rows) starting at tiles 0, 4, ..., the last moved back to end at the last one
// (rows it shares with the previous M tile are computed twice and dropped), so one load of the
// gradient serves every tap of the stage and no zero padding is multiplied.  A CTA walks its share
// of the pixel tiles (split K, one CTA per SM, 2-4 stages of 64-104 KB in flight) for the taps of
// its group (blockIdx.y) and adds its partial sums to dW with FP32 atomics.
constexpr int WG_M = 128;                          // rows of an M tile (TMEM lanes)
constexpr int WG_CHUNK = TC_BM * TC_KB * 2;        // one 128-pixel x 32-channel tile, 8 KB
constexpr int WG_SLACK = 16384;                    // keeps any reading of the descriptors inside the allocation
constexpr int HALO_ROW = 136;                      // pixels of a halo row x0 - 1 .. x0 + 134 (a multiple of 8)
constexpr int HALO_ROW_BYTES = 9216;               // HALO_ROW * 64 B rounded up to 1024 B
constexpr int HALO_STAGE = 3 * HALO_ROW_BYTES;     // three rows of one 32-channel block

struct WgArgs {
    float *gw;
    const __nv_bfloat16 *g;   // the output gradient, read by threads when Cout is not a multiple of 32
    int N, H, W, Cin, Cout;
    int BW, BH, tiles_x, tiles_y;
    int ntaps;              // taps of a CTA (9 or 3; blockIdx.y selects the group)
    int tg;                 // taps per stage (a divisor of ntaps)
    int tiles_per_cta, total_tiles;
    int xchunks, gchunks, stage_bytes, stages;
    int g_tma;              // 1: the gradient tiles come by TMA
    int ones;               // 1: a tile of ones after the input tiles yields the bias gradient
    float *gb;              // the bias gradient, accumulated when `ones`
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

// First 32-row tile of M tile mt over `chunks` tiles (the last M tile ends at the last tile).
__device__ __forceinline__ int ws_mstart(int mt, int chunks) { return chunks > 4 ? min(4 * mt, chunks - 4) : 0; }

// Byte offset of 16-byte unit u (0..3) of row r in a 64-byte-swizzled tile whose base is 512-B
// aligned: the unit index is XORed with bits 7..8 of the unswizzled offset, i.e. (r / 2) mod 4.
__device__ __forceinline__ unsigned sw64_off(int r, int u) { return (unsigned)(r * 64 + ((u ^ ((r >> 1) & 3)) << 4)); }

__device__ __forceinline__ unsigned short ld_bf16_bits(const __nv_bfloat16 *p)
{
    return __ldg(reinterpret_cast<const unsigned short *>(p));
}

// Unit U (channels 8U .. 8U + 7, zero past C) of pixel (n, py, px) of an NHWC tensor.
__device__ __forceinline__ uint4 pixel_unit(const __nv_bfloat16 *src, int C, int H, int W, int n, int py, int px, int U)
{
    const __nv_bfloat16 *p = src + (((size_t)n * H + py) * W + px) * C;
    if (C % 8 == 0) return __ldg(reinterpret_cast<const uint4 *>(p + U * 8));
    uint32_t v[4] = { 0u, 0u, 0u, 0u };
#pragma unroll
    for (int e = 0; e < 8; ++e)
        if (U * 8 + e < C) v[e >> 1] |= (uint32_t)ld_bf16_bits(p + U * 8 + e) << (16 * (e & 1));
    return make_uint4(v[0], v[1], v[2], v[3]);
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
    // the stage's M rows: the input tiles, then (ones) a tile whose every value is 1, so its rows
    // of dW^T are the sums of the gradient over the pixels, i.e. the bias gradient
    const int xall = a.xchunks + a.ones;
    const int npad = a.gchunks * TC_KB, mtiles = (xall + 3) / 4, blocks = a.ntaps / a.tg;
    const int used = blocks * mtiles * npad;
    const unsigned ncols = used <= 32 ? 32u : used <= 64 ? 64u : used <= 128 ? 128u : used <= 256 ? 256u : 512u;
    if (threadIdx.x == 0) {
        // full: the TMA producer's arrive (with the byte count), plus the two writer warps'
        for (int s = 0; s < a.stages; ++s) {
            mbar_init(smem_u32(&full[s]), a.g_tma ? 1 : 3);
            mbar_init(smem_u32(&empty[s]), 1);
        }
        mbar_init(smem_u32(done), 1);
        counts[0] = counts[1] = counts[2] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(ncols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (!a.g_tma) {   // the gradient units the writers never touch stay zero
        for (int s = 0; s < a.stages; ++s) {
            uint4 *z = reinterpret_cast<uint4 *>(smem + s * a.stage_bytes + xall * WG_CHUNK);
            for (int i = threadIdx.x; i < a.gchunks * WG_CHUNK / 16; i += blockDim.x) z[i] = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    if (a.ones) {     // bfloat16 1.0 in every element: the swizzle does not matter
        for (int s = 0; s < a.stages; ++s) {
            uint4 *o = reinterpret_cast<uint4 *>(smem + s * a.stage_bytes + a.xchunks * WG_CHUNK);
            for (int i = threadIdx.x; i < WG_CHUNK / 16; i += blockDim.x) o[i] = make_uint4(0x3F803F80u, 0x3F803F80u, 0x3F803F80u, 0x3F803F80u);
        }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = *tmem_slot;

    const int tap0 = blockIdx.y * a.ntaps;
    const int first = blockIdx.x * a.tiles_per_cta;
    const int ntiles = max(0, min(a.tiles_per_cta, a.total_tiles - first));
    const int iters = ntiles * blocks;
    const int per_img = a.tiles_x * a.tiles_y;
    const int kbx = a.Cin / TC_KB;

    if (warp == 0 && lane == 0) {              // producer: TMA loads of the shifted x tiles and the g tiles
        const unsigned bytes = (unsigned)((a.xchunks + (a.g_tma ? a.gchunks : 0)) * WG_CHUNK);
        for (int it = 0; it < iters; ++it) {
            const int s = it % a.stages;
            if (it >= a.stages && !mbar_wait(smem_u32(&empty[s]), (unsigned)((it / a.stages - 1) & 1))) {
                counts[2] = 1;
                break;
            }
            const int tile = first + it / blocks, b = it % blocks;
            const int n = tile / per_img, t2 = tile % per_img;
            const int y0 = (t2 / a.tiles_x) * a.BH, x0 = (t2 % a.tiles_x) * a.BW;
            unsigned char *st = smem + s * a.stage_bytes;
            const unsigned bar = smem_u32(&full[s]);
            mbar_expect_tx(bar, bytes);
            for (int t = 0; t < a.tg; ++t) {
                const int tap = tap0 + b * a.tg + t, dy = tap / 3 - 1, dx = tap % 3 - 1;
                for (int c = 0; c < kbx; ++c)
                    tma_load_4d(smem_u32(st + (t * kbx + c) * WG_CHUNK), &xmap, c * TC_KB, x0 + dx, y0 + dy, n, bar);
            }
            if (a.g_tma)
                for (int c = 0; c < a.gchunks; ++c)
                    tma_load_4d(smem_u32(st + (xall + c) * WG_CHUNK), &gmap, c * TC_KB, x0, y0, n, bar);
            counts[0] = it + 1;
        }
    } else if (warp == 1 && lane == 0) {       // MMA issuer
        const unsigned idesc = instr_desc_mn(npad);
        int it = 0;
        for (; it < iters; ++it) {
            const int s = it % a.stages;
            if (!mbar_wait(smem_u32(&full[s]), (unsigned)((it / a.stages) & 1))) {
                counts[2] = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const unsigned xbase = smem_u32(smem + s * a.stage_bytes), gbase = xbase + (unsigned)(xall * WG_CHUNK);
            const int b = it % blocks;
            const bool first_tile = it < blocks;
            for (int mt = 0; mt < mtiles; ++mt) {
                const unsigned abase = xbase + (unsigned)(ws_mstart(mt, xall) * WG_CHUNK);
                const unsigned dcol = tmem + (unsigned)((b * mtiles + mt) * npad);
#pragma unroll
                for (int k = 0; k < TC_BM / 16; ++k)   // K = 16 pixels per MMA: two 8-row groups, 1 KB on
                    umma(dcol, smem_desc_mn_sw64(abase + 1024 * k, WG_CHUNK), smem_desc_mn_sw64(gbase + 1024 * k, WG_CHUNK),
                         idesc, !(first_tile && k == 0));
            }
            umma_commit(smem_u32(&empty[s]));
            counts[1] = it + 1;
        }
        umma_commit(smem_u32(done));
    } else if (warp >= 2 && !a.g_tma) {        // writers of the narrow gradient tiles
        const int gunits = (a.Cout + 7) / 8;
        for (int it = 0; it < iters; ++it) {
            const int s = it % a.stages;
            bool ok = true;
            if (lane == 0 && it >= a.stages) ok = mbar_wait(smem_u32(&empty[s]), (unsigned)((it / a.stages - 1) & 1));
            if (!__shfl_sync(0xffffffffu, ok ? 1 : 0, 0)) {
                if (lane == 0) counts[2] = 1;
                break;
            }
            const int tile = first + it / blocks, n = tile / per_img, t2 = tile % per_img;
            const int y0 = (t2 / a.tiles_x) * a.BH, x0 = (t2 % a.tiles_x) * a.BW;
            unsigned char *gs = smem + s * a.stage_bytes + xall * WG_CHUNK;
            for (int q = threadIdx.x - 64; q < TC_BM * gunits; q += 64) {
                const int r = q & (TC_BM - 1), U = q >> 7;
                *reinterpret_cast<uint4 *>(gs + (U >> 2) * WG_CHUNK + sw64_off(r, U & 3)) =
                    pixel_unit(a.g, a.Cout, a.H, a.W, n, y0 + r / a.BW, x0 + r % a.BW, U);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full[s])) : "memory");
        }
    }
    if (!mbar_wait(smem_u32(done), 0)) counts[2] = 1;
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool valid = *((volatile int *)&counts[2]) == 0;
    if (iters > 0) {
        const int rows = 9 * a.Cin;
        for (int b = 0; b < blocks; ++b)
            for (int mt = 0; mt < mtiles; ++mt) {
                const int chunk = ws_mstart(mt, xall) + warp;   // warp w reads rows 32w .. 32w + 31
                if (chunk < 4 * mt || chunk >= xall) continue;   // computed by the previous M tile
                const bool bias = chunk == a.xchunks;   // the tile of ones: every row holds the bias gradient
                const int tap = tap0 + b * a.tg + chunk / kbx, row = tap * a.Cin + (chunk % kbx) * TC_KB + lane;
                for (int c0 = 0; c0 < npad; c0 += 16) {
                    unsigned v[16];
                    const unsigned taddr = tmem + ((unsigned)(warp * 32) << 16) + (unsigned)((b * mtiles + mt) * npad + c0);
                    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                                   "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                                 : "r"(taddr));
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    if (!valid) continue;
                    if (bias) {   // one lane, one tap group
                        if (lane == 0 && blockIdx.y == 0 && b == 0)
#pragma unroll
                            for (int e = 0; e < 16; ++e)
                                if (c0 + e < a.Cout) atomicAdd(&a.gb[c0 + e], __uint_as_float(v[e]));
                        continue;
                    }
#pragma unroll
                    for (int e = 0; e < 16; ++e)
                        if (c0 + e < a.Cout) atomicAdd(&a.gw[(size_t)(c0 + e) * rows + row], __uint_as_float(v[e]));
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

// ---- weight gradient with halo rows (W a multiple of 128) ------------------------------------
// dW^T as in k_wgrad_tc, but a pixel tile is 128 pixels of one image row and its input comes as the
// three 136-pixel halo rows (x0 - 1 .. x0 + 134) of each 32-channel block, as in k_conv_halo_tc.
// An M tile is (dy, channel block): its four 32-row chunks are the taps dx = -1, 0, +1 (and a
// fourth, dropped) of that halo row, i.e. the same buffer read from 64-byte offsets: the MN-major
// descriptor's leading byte offset is 64 B (one pixel row), the stride byte offset 512 B per 8
// pixels, and the 64-byte swizzle follows the address bits.  Per pixel tile 3 x Cin / 32 halo rows
// (8.5 KB each) and the gradient tile instead of nine shifted tiles per channel block.
struct WhArgs {
    float *gw;
    const __nv_bfloat16 *g;   // read by the writer warps when Cout is not a multiple of 32
    int N, H, W, Cin, Cout;
    int tiles_x, total_tiles, tiles_per_cta;
    int kbx, gchunks, stage_bytes, stages;
    int g_tma;
    int *err;
};

__global__ void __launch_bounds__(128, 1)
k_wgrad_halo_tc(const __grid_constant__ CUtensorMap hmap, const __grid_constant__ CUtensorMap gmap, WhArgs a)
{
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    unsigned char *smem = tc_smem_raw + ((1024 - (smem_u32(tc_smem_raw) & 1023)) & 1023);
    unsigned long long *bars = reinterpret_cast<unsigned long long *>(smem + a.stages * a.stage_bytes + WG_SLACK);
    unsigned long long *full = bars, *empty = bars + a.stages, *done = bars + 2 * a.stages;
    unsigned *tmem_slot = reinterpret_cast<unsigned *>(bars + 2 * a.stages + 1);
    int *counts = reinterpret_cast<int *>(tmem_slot + 1);   // [0] issued, [1] consumed, [2] failed

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int npad = a.gchunks * TC_KB, mtiles = 3 * a.kbx, used = mtiles * npad;
    const int rows_bytes = 3 * a.kbx * HALO_ROW_BYTES;   // halo rows of the stage: [dy][kb]
    const unsigned ncols = used <= 32 ? 32u : used <= 64 ? 64u : used <= 128 ? 128u : used <= 256 ? 256u : 512u;
    if (threadIdx.x == 0) {
        for (int s = 0; s < a.stages; ++s) {
            mbar_init(smem_u32(&full[s]), a.g_tma ? 1 : 3);
            mbar_init(smem_u32(&empty[s]), 1);
        }
        mbar_init(smem_u32(done), 1);
        counts[0] = counts[1] = counts[2] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(ncols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (!a.g_tma) {   // the gradient units the writers never touch stay zero
        for (int s = 0; s < a.stages; ++s) {
            uint4 *z = reinterpret_cast<uint4 *>(smem + s * a.stage_bytes + rows_bytes);
            for (int i = threadIdx.x; i < a.gchunks * WG_CHUNK / 16; i += blockDim.x) z[i] = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = *tmem_slot;

    const int first = blockIdx.x * a.tiles_per_cta;
    const int iters = max(0, min(a.tiles_per_cta, a.total_tiles - first));
    const int per_img = a.tiles_x * a.H;

    if (warp == 0 && lane == 0) {              // producer: the halo rows and the g tiles of each pixel tile
        const unsigned bytes = (unsigned)(rows_bytes / HALO_ROW_BYTES * HALO_ROW * 64 + (a.g_tma ? a.gchunks * WG_CHUNK : 0));
        for (int it = 0; it < iters; ++it) {
            const int s = it % a.stages;
            if (it >= a.stages && !mbar_wait(smem_u32(&empty[s]), (unsigned)((it / a.stages - 1) & 1))) {
                counts[2] = 1;
                break;
            }
            const int tile = first + it, n = tile / per_img, r = tile % per_img;
            const int y0 = r / a.tiles_x, x0 = (r % a.tiles_x) * TC_BM;
            unsigned char *st = smem + s * a.stage_bytes;
            const unsigned bar = smem_u32(&full[s]);
            mbar_expect_tx(bar, bytes);
            for (int dy = 0; dy < 3; ++dy)
                for (int kb = 0; kb < a.kbx; ++kb)
                    tma_load_4d(smem_u32(st + (dy * a.kbx + kb) * HALO_ROW_BYTES), &hmap, kb * TC_KB, x0 - 1, y0 + dy - 1,
                                n, bar);
            if (a.g_tma)
                for (int c = 0; c < a.gchunks; ++c)
                    tma_load_4d(smem_u32(st + rows_bytes + c * WG_CHUNK), &gmap, c * TC_KB, x0, y0, n, bar);
            counts[0] = it + 1;
        }
    } else if (warp == 1 && lane == 0) {       // MMA issuer
        const unsigned idesc = instr_desc_mn(npad);
        int it = 0;
        for (; it < iters; ++it) {
            const int s = it % a.stages;
            if (!mbar_wait(smem_u32(&full[s]), (unsigned)((it / a.stages) & 1))) {
                counts[2] = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const unsigned rbase = smem_u32(smem + s * a.stage_bytes), gbase = rbase + (unsigned)rows_bytes;
            for (int mt = 0; mt < mtiles; ++mt) {
                const unsigned abase = rbase + (unsigned)(mt * HALO_ROW_BYTES);
                const unsigned dcol = tmem + (unsigned)(mt * npad);
#pragma unroll
                for (int k = 0; k < TC_BM / 16; ++k)   // K = 16 pixels per MMA: 1 KB on in both operands
                    umma(dcol, smem_desc_mn_sw64(abase + 1024 * k, 64), smem_desc_mn_sw64(gbase + 1024 * k, WG_CHUNK),
                         idesc, !(it == 0 && k == 0));
            }
            umma_commit(smem_u32(&empty[s]));
            counts[1] = it + 1;
        }
        umma_commit(smem_u32(done));
    } else if ((warp == 2 || warp == 3) && !a.g_tma) {   // writers of the narrow gradient tiles
        const int gunits = (a.Cout + 7) / 8;
        for (int it = 0; it < iters; ++it) {
            const int s = it % a.stages;
            bool ok = true;
            if (lane == 0 && it >= a.stages) ok = mbar_wait(smem_u32(&empty[s]), (unsigned)((it / a.stages - 1) & 1));
            if (!__shfl_sync(0xffffffffu, ok ? 1 : 0, 0)) {
                if (lane == 0) counts[2] = 1;
                break;
            }
            const int tile = first + it, n = tile / per_img, r = tile % per_img;
            const int y0 = r / a.tiles_x, x0 = (r % a.tiles_x) * TC_BM;
            unsigned char *gs = smem + s * a.stage_bytes + rows_bytes;
            for (int q = threadIdx.x - 64; q < TC_BM * gunits; q += 64) {
                const int rr = q & (TC_BM - 1), U = q >> 7;
                *reinterpret_cast<uint4 *>(gs + (U >> 2) * WG_CHUNK + sw64_off(rr, U & 3)) =
                    pixel_unit(a.g, a.Cout, a.H, a.W, n, y0, x0 + rr, U);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full[s])) : "memory");
        }
    }
    if (!mbar_wait(smem_u32(done), 0)) counts[2] = 1;
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool valid = *((volatile int *)&counts[2]) == 0;
    if (iters > 0 && warp < 3) {   // warp w: chunk w of each M tile, tap dx = w - 1 (warp 3: the dropped chunk)
        const int rows = 9 * a.Cin;
        for (int mt = 0; mt < mtiles; ++mt) {
            const int dy = mt / a.kbx, kb = mt % a.kbx;
            const int row = (dy * 3 + warp) * a.Cin + kb * TC_KB + lane;
            for (int c0 = 0; c0 < npad; c0 += 16) {
                unsigned v[16];
                const unsigned taddr = tmem + ((unsigned)(warp * 32) << 16) + (unsigned)(mt * npad + c0);
                asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                             : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                               "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                             : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (!valid) continue;
#pragma unroll
                for (int e = 0; e < 16; ++e)
                    if (c0 + e < a.Cout) atomicAdd(&a.gw[(size_t)(c0 + e) * rows + row], __uint_as_float(v[e]));
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

// ---- layers with a narrow side ----------------------------------------------------------------
// A pixel of a tensor with fewer than 8 channels (the operator's 4-channel input, its 3-channel
// output) is under TMA's 16-byte minimum row, so these layers' operands are written into shared
// memory by the CTA's threads, in the layouts the TMA tiles above have (rows of 64 bytes, 16-byte
// units swizzled in groups of 8 rows), and fed to the same tcgen05.mma forms:
//  * forward (and, on the flipped weights, the input gradient) with 9 * Cin <= 64: M = 128 pixels,
//    K = the (tap, ci) columns of the im2col tile padded to 32 or 64, N = Cout padded to 16;
//  * weight gradient with Cin <= 32: M = Cout padded to 128 (the gradient tile), N = the 9 * Cin
//    (tap, ci) columns of the im2col tile, K = the pixels, both MN-major as in k_wgrad_tc.
constexpr int SM_BUILD = 128;      // threads of a CTA, all of which write operand tiles

// Unit U (columns 8U .. 8U + 7) of the im2col row of pixel (n, py, px): column c = tap * C + ch holds
// src[n][py + s * (tap / 3 - 1)][px + s * (tap % 3 - 1)][ch] (zero outside the image and for
// c >= 9 * C); s = 1 for the forward convolution.
__device__ __forceinline__ uint4 im2col_unit(const __nv_bfloat16 *src, int C, int H, int W, int n, int py, int px,
                                             int U)
{
    uint32_t v[4] = { 0u, 0u, 0u, 0u };
    const int c0 = U * 8;
    if (C % 8 == 0) {   // one tap, eight consecutive channels: a 16-byte load
        const int tap = c0 / C, ch = c0 - tap * C;
        const int sy = py + tap / 3 - 1, sx = px + tap % 3 - 1;
        if (tap < 9 && sy >= 0 && sy < H && sx >= 0 && sx < W)
            return __ldg(reinterpret_cast<const uint4 *>(src + (((size_t)n * H + sy) * W + sx) * C + ch));
        return make_uint4(0u, 0u, 0u, 0u);
    }
    if (C == 4) {       // two taps of four channels: two 8-byte loads
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int tap = 2 * U + h;
            const int sy = py + tap / 3 - 1, sx = px + tap % 3 - 1;
            if (tap < 9 && sy >= 0 && sy < H && sx >= 0 && sx < W) {
                const uint2 q = __ldg(reinterpret_cast<const uint2 *>(src + (((size_t)n * H + sy) * W + sx) * 4));
                v[2 * h] = q.x;
                v[2 * h + 1] = q.y;
            }
        }
        return make_uint4(v[0], v[1], v[2], v[3]);
    }
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const int c = c0 + e, tap = c / C, ch = c - tap * C;
        const int sy = py + tap / 3 - 1, sx = px + tap % 3 - 1;
        if (tap < 9 && sy >= 0 && sy < H && sx >= 0 && sx < W)
            v[e >> 1] |= (uint32_t)ld_bf16_bits(src + (((size_t)n * H + sy) * W + sx) * C + ch) << (16 * (e & 1));
    }
    return make_uint4(v[0], v[1], v[2], v[3]);
}

struct SmallArgs {
    const __nv_bfloat16 *x;     // forward: input [N,H,W,Cin]; weight gradient: input
    const __nv_bfloat16 *w;     // forward: weights [Cout][9 * Cin]
    const __nv_bfloat16 *g;     // weight gradient: gradient of the output [N,H,W,Cout]
    const float *bias;          // forward, may be null
    __nv_bfloat16 *y;           // forward: output [N,H,W,Cout]
    float *gw;                  // weight gradient: [Cout][9 * Cin], accumulated
    int N, H, W, Cin, Cout, npad, relu;
    int BW, BH, tiles_x, tiles_y;
    int kchunks;                // forward: 32-column chunks of the im2col tile (1 or 2)
    int bchunks;                // weight gradient: 32-column chunks of the im2col tile (<= 9)
    int tiles_per_cta, total_tiles, stage_bytes;
    int *err;
};

// Forward convolution of a narrow input: one 128-pixel tile per CTA; the threads write the im2col
// tile (K-major: row = pixel, kchunks chunks of 32 columns) and the weights (row = output channel),
// one thread issues kchunks * 2 MMAs (K = 16 each) into a TMEM accumulator of npad columns.
__global__ void __launch_bounds__(SM_BUILD, 8) k_conv_small_tc(SmallArgs a)
{
    __shared__ float s_bias[128];
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    unsigned char *smem = tc_smem_raw + ((1024 - (smem_u32(tc_smem_raw) & 1023)) & 1023);
    unsigned char *As = smem, *Bs = smem + a.kchunks * WG_CHUNK;
    unsigned long long *done = reinterpret_cast<unsigned long long *>(Bs + a.kchunks * a.npad * 64);
    unsigned *tmem_slot = reinterpret_cast<unsigned *>(done + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned ncols = a.npad <= 32 ? 32u : (a.npad <= 64 ? 64u : 128u);
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(done), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(ncols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    stage_bias(s_bias, a.bias, a.Cout, a.npad);
    const int per_img = a.tiles_x * a.tiles_y;
    const int n = blockIdx.x / per_img, t2 = blockIdx.x % per_img;
    const int y0 = (t2 / a.tiles_x) * a.BH, x0 = (t2 % a.tiles_x) * a.BW;
    {   // A: thread r writes row r (pixel r of the tile)
        const int r = threadIdx.x, px = x0 + r % a.BW, py = y0 + r / a.BW;
        for (int c = 0; c < a.kchunks; ++c) {
            uint4 u[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) u[k] = im2col_unit(a.x, a.Cin, a.H, a.W, n, py, px, c * 4 + k);
#pragma unroll
            for (int k = 0; k < 4; ++k) *reinterpret_cast<uint4 *>(As + c * WG_CHUNK + sw64_off(r, k)) = u[k];
        }
    }
    const int K = 9 * a.Cin;
    for (int i = threadIdx.x; i < a.kchunks * a.npad * 4; i += SM_BUILD) {   // B: row j = output channel j
        const int c = i / (a.npad * 4), rem = i - c * a.npad * 4, j = rem >> 2, k = rem & 3;
        uint32_t v[4] = { 0u, 0u, 0u, 0u };
        if (j < a.Cout) {
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int col = c * 32 + k * 8 + e;
                if (col < K) v[e >> 1] |= (uint32_t)ld_bf16_bits(a.w + (size_t)j * K + col) << (16 * (e & 1));
            }
        }
        *reinterpret_cast<uint4 *>(Bs + c * a.npad * 64 + sw64_off(j, k)) = make_uint4(v[0], v[1], v[2], v[3]);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // the tiles are read by the tensor cores
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = *tmem_slot;
    if (threadIdx.x == 0) {
        const unsigned idesc = instr_desc(a.npad);
        const unsigned abase = smem_u32(As), bbase = smem_u32(Bs);
        for (int c = 0; c < a.kchunks; ++c)
#pragma unroll
            for (int k = 0; k < 2; ++k)
                umma(tmem, smem_desc_sw64(abase + c * WG_CHUNK + 32 * k), smem_desc_sw64(bbase + c * a.npad * 64 + 32 * k),
                     idesc, c > 0 || k > 0);
        umma_commit(smem_u32(done));
    }
    const bool valid = mbar_wait(smem_u32(done), 0);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int row = warp * 32 + lane;
    const int px = x0 + row % a.BW, py = y0 + row / a.BW;
    for (int c0 = 0; c0 < a.npad; c0 += 16) {
        unsigned v[16];
        const unsigned taddr = tmem + ((unsigned)(warp * 32) << 16) + (unsigned)c0;
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                     : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                       "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                     : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (!valid || py >= a.H || px >= a.W) continue;
        store_row16(a.y + (((size_t)n * a.H + py) * a.W + px) * a.Cout, c0, a.Cout, v, s_bias, a.relu);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0 && !valid) {
        atomicExch(a.err, 1);
        mbar_wait(smem_u32(done), 0);
    }
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
    }
}

// Weight gradient with a narrow side, as dW^T: M = the 9 * Cin (tap, ci) columns of the input's
// im2col tile, N = Cout padded to 32 * gchunks, K = the pixels; both operands MN-major (a row is one
// pixel holding 32 consecutive M or N elements, chunks 8 KB apart).  The M rows are covered by
// tiles of four chunks (128 rows) starting at chunks 0, 4, ..., the last one moved back to end at
// the last chunk (its rows already covered by the previous tile are computed twice and dropped),
// so no zero chunks are multiplied once there are four.  A CTA walks its share of the 128-pixel
// tiles through two stages: all threads load the tile's units (ten per thread in flight) and write
// them swizzled, one thread issues the MMAs and releases the stage with tcgen05.commit, so writing
// tile j + 1 overlaps the MMAs of tile j.  Four warps then read the accumulators (warp w: chunk
// w of an M tile, lane = (tap, ci) column) and add them to dW[co][(tap, ci)] with FP32 atomics.
constexpr int WS_THREADS = 256, WS_BATCH = 10;

__global__ void __launch_bounds__(WS_THREADS, 2) k_wgrad_small_tc(SmallArgs a)
{
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    unsigned char *smem = tc_smem_raw + ((1024 - (smem_u32(tc_smem_raw) & 1023)) & 1023);
    unsigned long long *bars = reinterpret_cast<unsigned long long *>(smem + 2 * a.stage_bytes + WG_SLACK);
    unsigned long long *empty = bars, *done = bars + 2;
    unsigned *tmem_slot = reinterpret_cast<unsigned *>(bars + 3);
    int *failed = reinterpret_cast<int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cols = 9 * a.Cin;                         // (tap, ci) columns
    const int xchunks = a.bchunks, xalloc = max(xchunks, 4), mtiles = (xchunks + 3) / 4;
    const int gchunks = (a.Cout + TC_KB - 1) / TC_KB, npad = gchunks * TC_KB;
    const int used = mtiles * npad;
    const unsigned ncols = used <= 32 ? 32u : used <= 64 ? 64u : used <= 128 ? 128u : used <= 256 ? 256u : 512u;
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(&empty[0]), 1);
        mbar_init(smem_u32(&empty[1]), 1);
        mbar_init(smem_u32(done), 1);
        *failed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(ncols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    for (int i = threadIdx.x; i < 2 * a.stage_bytes / 16; i += WS_THREADS)   // units never written stay zero
        reinterpret_cast<uint4 *>(smem)[i] = make_uint4(0u, 0u, 0u, 0u);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = *tmem_slot;

    const int first = blockIdx.x * a.tiles_per_cta;
    const int ntiles = max(0, min(a.tiles_per_cta, a.total_tiles - first));
    const int per_img = a.tiles_x * a.tiles_y;
    const int gunits = (a.Cout + 7) / 8, xunits = (cols + 7) / 8;
    const int units = TC_BM * (gunits + xunits);        // (pixel, unit) pairs of a tile
    const unsigned idesc = instr_desc_mn(npad);
    for (int j = 0; j < ntiles; ++j) {
        const int s = j & 1;
        if (j >= 2 && threadIdx.x == 0 && !mbar_wait(smem_u32(&empty[s]), (unsigned)(((j >> 1) - 1) & 1))) *failed = 1;
        __syncthreads();
        if (*((volatile int *)failed)) break;
        const int tile = first + j, n = tile / per_img, t2 = tile % per_img;
        const int py0 = (t2 / a.tiles_x) * a.BH, px0 = (t2 % a.tiles_x) * a.BW;
        unsigned char *Xs = smem + s * a.stage_bytes, *Gs = Xs + xalloc * WG_CHUNK;
        for (int q0 = threadIdx.x; q0 < units; q0 += WS_THREADS * WS_BATCH) {
            uint4 u[WS_BATCH];
#pragma unroll
            for (int k = 0; k < WS_BATCH; ++k) {   // unit q: pixel q % 128, unit q / 128 (gradient units first)
                const int q = q0 + k * WS_THREADS;
                if (q >= units) break;
                const int r = q & (TC_BM - 1), U = q >> 7, py = py0 + r / a.BW, px = px0 + r % a.BW;
                u[k] = U < gunits ? pixel_unit(a.g, a.Cout, a.H, a.W, n, py, px, U)
                                  : im2col_unit(a.x, a.Cin, a.H, a.W, n, py, px, U - gunits);
            }
#pragma unroll
            for (int k = 0; k < WS_BATCH; ++k) {
                const int q = q0 + k * WS_THREADS;
                if (q >= units) break;
                const int r = q & (TC_BM - 1), U = q >> 7, V = U < gunits ? U : U - gunits;
                unsigned char *base = U < gunits ? Gs : Xs;
                *reinterpret_cast<uint4 *>(base + (V >> 2) * WG_CHUNK + sw64_off(r, V & 3)) = u[k];
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const unsigned xbase = smem_u32(Xs), gbase = smem_u32(Gs);
#pragma unroll 1
            for (int mt = 0; mt < mtiles; ++mt) {
                const unsigned abase = xbase + (unsigned)(ws_mstart(mt, xchunks) * WG_CHUNK);
#pragma unroll
                for (int k = 0; k < TC_BM / 16; ++k)   // K = 16 pixels per MMA: two 8-row groups, 1 KB on
                    umma(tmem + (unsigned)(mt * npad), smem_desc_mn_sw64(abase + 1024 * k, WG_CHUNK),
                         smem_desc_mn_sw64(gbase + 1024 * k, WG_CHUNK), idesc, j > 0 || k > 0);
            }
            umma_commit(smem_u32(&empty[s]));
        }
    }
    if (threadIdx.x == 0) umma_commit(smem_u32(done));   // arrives when every issued MMA has completed
    if (!mbar_wait(smem_u32(done), 0)) *failed = 1;
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool valid = *((volatile int *)failed) == 0;
    if (ntiles > 0 && warp < 4) {
        for (int mt = 0; mt < mtiles; ++mt) {
            const int chunk = ws_mstart(mt, xchunks) + warp;
            if (chunk < 4 * mt || chunk >= xchunks) continue;   // computed by the previous tile / padding
            const int col = chunk * TC_KB + lane;
            for (int c0 = 0; c0 < npad; c0 += 16) {
                unsigned v[16];
                const unsigned taddr = tmem + ((unsigned)(warp * 32) << 16) + (unsigned)(mt * npad + c0);
                asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                             : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                               "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                             : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (!valid || col >= cols) continue;
#pragma unroll
                for (int e = 0; e < 16; ++e)
                    if (c0 + e < a.Cout) atomicAdd(&a.gw[(size_t)(c0 + e) * cols + col], __uint_as_float(v[e]));
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0 && !valid) {
        atomicExch(a.err, 1);
        mbar_wait(smem_u32(done), 0);
    }
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
    }
}

// ---- forward convolution with halo rows (W a multiple of 128) ---------------------------------
// A tile is 128 pixels of one image row.  Instead of nine shifted input tiles per 32-channel block,
// the three input rows y0 - 1, y0, y0 + 1 are loaded once as halo rows of 136 pixels (x0 - 1 ..
// x0 + 134, TMA zero fill outside the image), and tap (dy, dx) reads the 128 rows of halo row dy + 1
// that start at pixel dx + 1, i.e. a descriptor start address 64 * (dx + 1) bytes into the row
// buffer: 26 KB per block instead of 72 KB.  The tensor cores apply the 64-byte swizzle to the
// address bits, as the TMA wrote the rows, so such a start needs no base offset in the descriptor
// (measured: with the base offset set from the start address the results are wrong).  The weights of the whole layer stay in shared memory
// (loaded once per CTA) and CTAs are persistent (one per SM).  A CTA's tiles alternate between two
// pipelines, each with its own ring of stages, its own MMA-issuing thread (warps 1 and 6) and two
// TMEM accumulators: one thread issues a tcgen05.mma about every 100 cycles (measured), so a
// single issuer leaves the tensor pipe idle three quarters of the time at N <= 128.  Warp 0 loads
// for both, warps 2..5 drain the accumulators in tile order (bias, ReLU, BF16 stores) while the
// next tiles accumulate.
constexpr int HALO_MAX_STAGES = 3;            // per pipeline

struct HaloArgs {
    __nv_bfloat16 *y;
    const float *bias;      // may be null
    int N, H, W, Cin, Cout, npad, relu;
    int tiles_x, tiles;     // 128-pixel tiles per image row, in all
    int kblocks, stages, w_bytes;
    int *err;
};


__global__ void __launch_bounds__(224, 1)
k_conv_halo_tc(const __grid_constant__ CUtensorMap hmap, const __grid_constant__ CUtensorMap wmap, HaloArgs a)
{
    __shared__ float s_bias[128];
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    unsigned char *smem = tc_smem_raw + ((1024 - (smem_u32(tc_smem_raw) & 1023)) & 1023);
    const int S = a.stages, NS = 2 * S;       // stages per pipeline, in all
    unsigned char *wts = smem, *rows = smem + a.w_bytes;
    unsigned long long *bars = reinterpret_cast<unsigned long long *>(rows + NS * HALO_STAGE);
    unsigned long long *full = bars, *empty = bars + NS, *tfull = bars + 2 * NS, *tempty = tfull + 4,
                       *wfull = tempty + 4, *done = wfull + 1;
    unsigned *tmem_slot = reinterpret_cast<unsigned *>(done + 2);
    int *counts = reinterpret_cast<int *>(tmem_slot + 1);   // [p] issued, [2 + p] consumed, [4] failed
    volatile int *failed = &counts[4];

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned ncols = 4 * a.npad <= 64 ? 64u : 4 * a.npad <= 128 ? 128u : 4 * a.npad <= 256 ? 256u : 512u;
    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) { mbar_init(smem_u32(&full[s]), 1); mbar_init(smem_u32(&empty[s]), 1); }
        for (int b = 0; b < 4; ++b) { mbar_init(smem_u32(&tfull[b]), 1); mbar_init(smem_u32(&tempty[b]), 4); }
        mbar_init(smem_u32(wfull), 1);
        mbar_init(smem_u32(&done[0]), 1);
        mbar_init(smem_u32(&done[1]), 1);
        for (int k = 0; k < 5; ++k) counts[k] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(ncols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    stage_bias(s_bias, a.bias, a.Cout, a.npad);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = *tmem_slot;
    const int per_img = a.tiles_x * a.H;
    const unsigned wchunk = (unsigned)a.npad * 64u;
    // the CTA's tiles t_i = blockIdx.x + i * gridDim.x alternate between the pipelines: p = i & 1
    const int ntiles = a.tiles > (int)blockIdx.x ? (a.tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

    if (warp == 0 && lane == 0) {              // producer: the weights once, then the halo rows in tile order
        mbar_expect_tx(smem_u32(wfull), (unsigned)(9 * a.kblocks) * wchunk);
        for (int kb = 0; kb < a.kblocks; ++kb)
            for (int tap = 0; tap < 9; ++tap)
                tma_load_3d(smem_u32(wts + (kb * 9 + tap) * wchunk), &wmap, kb * TC_KB, tap, 0, smem_u32(wfull));
        for (int i = 0; i < ntiles && !*failed; ++i) {
            const int t = blockIdx.x + i * gridDim.x, p = i & 1, ip = i >> 1;
            const int n = t / per_img, r = t % per_img, y0 = r / a.tiles_x, x0 = (r % a.tiles_x) * TC_BM;
            for (int kb = 0; kb < a.kblocks; ++kb) {
                const int itp = ip * a.kblocks + kb, s = p * S + itp % S;
                if (itp >= S && !mbar_wait(smem_u32(&empty[s]), (unsigned)((itp / S - 1) & 1))) {
                    *failed = 1;
                    break;
                }
                const unsigned bar = smem_u32(&full[s]);
                mbar_expect_tx(bar, 3u * HALO_ROW * 64u);
                for (int dy = 0; dy < 3; ++dy)
                    tma_load_4d(smem_u32(rows + s * HALO_STAGE + dy * HALO_ROW_BYTES), &hmap, kb * TC_KB, x0 - 1,
                                y0 + dy - 1, n, bar);
                counts[p] = itp + 1;
            }
        }
    } else if ((warp == 1 || warp == 6) && lane == 0) {   // MMA issuers, one per pipeline
        const int p = warp == 1 ? 0 : 1;
        const unsigned idesc = instr_desc(a.npad);
        if (!mbar_wait(smem_u32(wfull), 0)) *failed = 1;
        const uint64_t bstep = wchunk >> 4;
        for (int ip = 0; 2 * ip + p < ntiles && !*failed; ++ip) {
            const int b = ip & 1, acc = p * 2 + b;
            if (ip >= 2 && !mbar_wait(smem_u32(&tempty[acc]), (unsigned)(((ip >> 1) - 1) & 1))) {
                *failed = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const unsigned d = tmem + (unsigned)(acc * a.npad);
            for (int kb = 0; kb < a.kblocks; ++kb) {
                const int itp = ip * a.kblocks + kb, s = p * S + itp % S;
                if (!mbar_wait(smem_u32(&full[s]), (unsigned)((itp / S) & 1))) {
                    *failed = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                // descriptors of the stage's first row and the block's first tap; the others differ only
                // in the start-address field (bytes / 16, no carry below 256 KB): one add per operand
                const uint64_t ad0 = smem_desc_sw64(smem_u32(rows + s * HALO_STAGE));
                const uint64_t bd0 = smem_desc_sw64(smem_u32(wts + kb * 9 * wchunk));
#pragma unroll
                for (int tap = 0; tap < 9; ++tap)
#pragma unroll
                    for (int k = 0; k < TC_KB / 16; ++k)
                        umma(d, ad0 + (uint64_t)(((tap / 3) * HALO_ROW_BYTES + (tap % 3) * 64 + 32 * k) >> 4),
                             bd0 + (uint64_t)tap * bstep + (uint64_t)(2 * k), idesc, kb > 0 || tap > 0 || k > 0);
                umma_commit(smem_u32(&empty[s]));
                counts[2 + p] = itp + 1;
            }
            umma_commit(smem_u32(&tfull[acc]));
        }
        umma_commit(smem_u32(&done[p]));
    } else if (warp >= 2 && warp <= 5) {       // epilogue: TMEM lanes 32 * (warp % 4) .., tiles in order
        const int sub = warp & 3, row = sub * 32 + lane;
        for (int i = 0; i < ntiles; ++i) {
            const int t = blockIdx.x + i * gridDim.x, p = i & 1, ip = i >> 1, acc = p * 2 + (ip & 1);
            bool ok = true;
            if (lane == 0) ok = mbar_wait(smem_u32(&tfull[acc]), (unsigned)((ip >> 1) & 1));
            if (!__shfl_sync(0xffffffffu, ok ? 1 : 0, 0)) {
                if (lane == 0) *failed = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int n = t / per_img, r = t % per_img, y0 = r / a.tiles_x, px = (r % a.tiles_x) * TC_BM + row;
            __nv_bfloat16 *out = a.y + (((size_t)n * a.H + y0) * a.W + px) * a.Cout;
            for (int c0 = 0; c0 < a.npad; c0 += 32) {   // two 16-column loads per wait (npad: a multiple of 16)
                unsigned v[2][16];
                const unsigned taddr = tmem + ((unsigned)(sub * 32) << 16) + (unsigned)(acc * a.npad + c0);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    if (c0 + 16 * h >= a.npad) break;
                    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                                 : "=r"(v[h][0]), "=r"(v[h][1]), "=r"(v[h][2]), "=r"(v[h][3]), "=r"(v[h][4]), "=r"(v[h][5]),
                                   "=r"(v[h][6]), "=r"(v[h][7]), "=r"(v[h][8]), "=r"(v[h][9]), "=r"(v[h][10]), "=r"(v[h][11]),
                                   "=r"(v[h][12]), "=r"(v[h][13]), "=r"(v[h][14]), "=r"(v[h][15])
                                 : "r"(taddr + 16u * h));
                }
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                store_row16(out, c0, a.Cout, v[0], s_bias, a.relu);
                if (c0 + 16 < a.npad) store_row16(out, c0 + 16, a.Cout, v[1], s_bias, a.relu);
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[acc])) : "memory");
        }
    }
    if (threadIdx.x == 0) {   // every issued MMA has completed (each issuer commits its own)
        if (!mbar_wait(smem_u32(&done[0]), 0) || !mbar_wait(smem_u32(&done[1]), 0)) *failed = 1;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0 && *failed) {
        atomicExch(a.err, 1);
        // after a failed wait: the weights and the halo rows still in flight, each bounded
        mbar_wait(smem_u32(wfull), 0);
        for (int p = 0; p < 2; ++p)
            for (int itp = counts[2 + p]; itp < counts[p]; ++itp)
                mbar_wait(smem_u32(&full[p * S + itp % S]), (unsigned)((itp / S) & 1));
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
static bool tiles_exactly(int H, int W)
{
    if (H < 1 || W < 1) return false;
    if (W % TC_BM == 0) return true;
    if (TC_BM % W != 0) return false;
    return H % (TC_BM / W) == 0;
}

bool plbm_nn_tc_supported(int H, int W, int Cin, int Cout)
{
    if (Cin % TC_KB != 0 || Cin > 4096 || Cout < 1 || Cout > 128) return false;
    return tiles_exactly(H, W);
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
    // rows of 128 pixels: the halo-row kernel, when the layer's weights and two stages fit
    const int kblocks = Cin / TC_KB;
    const int w_bytes = 9 * kblocks * npad * 64;
    const int halo_budget = 227 * 1024 - 1024 - 512 - 1024;   // less alignment, barriers, the static bias array
    const int hfit = (halo_budget - w_bytes) / (2 * HALO_STAGE);   // stages per pipeline (two pipelines)
    const int hstages = hfit < HALO_MAX_STAGES ? hfit : HALO_MAX_STAGES;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    // each persistent CTA loads the whole layer's weights first: worth it from four tiles per SM on
    if (W % TC_BM == 0 && hstages >= 1 && N * H * (W / TC_BM) >= 4 * sms) {
        CUtensorMap hmap;
        const cuuint64_t dims[4] = { (cuuint64_t)Cin, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N };
        const cuuint64_t strides[3] = { (cuuint64_t)Cin * 2, (cuuint64_t)W * Cin * 2, (cuuint64_t)H * W * Cin * 2 };
        const cuuint32_t box[4] = { TC_KB, HALO_ROW, 1, 1 };
        const cuuint32_t es[4] = { 1, 1, 1, 1 };
        if (enc(&hmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(x), dims, strides, box, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return PLBM_ERR_ARGUMENT;
        const int smem = w_bytes + 2 * hstages * HALO_STAGE + 1024 + 512;
        static int halo_attr = 0;
        {
            std::lock_guard<std::mutex> g(mu);
            if (smem > halo_attr) {
                if (cudaFuncSetAttribute(k_conv_halo_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
                    return PLBM_ERR_CUDA;
                halo_attr = smem;
            }
        }
        HaloArgs h{ (__nv_bfloat16 *)y, bias, N, H, W, Cin, Cout, npad, relu, W / TC_BM, N * H * (W / TC_BM),
                    kblocks, hstages, w_bytes, err };
        k_conv_halo_tc<<<h.tiles < sms ? h.tiles : sms, 224, smem, s>>>(hmap, wmap, h);
        return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
    }
    // stages sized by the padded output channels, so narrow layers fit more CTAs per SM
    const int stage = TC_A_BYTES + (npad * TC_KB * 2 + 1023) / 1024 * 1024;
    TcArgs a{ (__nv_bfloat16 *)y, bias, N, H, W, Cin, Cout, npad, relu, BW, BH, W / BW, H / BH, stage, err };
    const int tiles = N * a.tiles_x * a.tiles_y;
    k_conv_tc<<<tiles, 128, TC_STAGES * stage + 1024 + 256, s>>>(xmap, wmap, a);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

// The weight gradient runs on the TMA-fed tensor-core kernel for Cin a multiple of 32 up to 128,
// Cout up to 128 (TMA gradient tiles for multiples of 32, written by two warps otherwise) and the
// image tilings of the forward kernel.
bool plbm_nn_tc_wgrad_supported(int H, int W, int Cin, int Cout)
{
    if (Cin % TC_KB != 0 || Cin < TC_KB || Cin > 128 || Cout < 1 || Cout > WG_M) return false;
    return tiles_exactly(H, W);
}

// gw[co][tap][ci] += sum_p g[p][co] x[p + tap][ci] on the tensor cores (x, g NHWC BF16, gw FP32); with
// gb, also gb[co] += sum_p g[p][co] where a tile of ones fits the stage without another M tile
// (*bias_done = 1; the caller then runs no bias kernel).
int plbm_nn_tc_wgrad(const void *x, const void *g, float *gw, float *gb, int N, int H, int W, int Cin, int Cout,
                     int *bias_done, cudaStream_t s)
{
    if (bias_done) *bias_done = 0;
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    int *err = error_flag();
    if (!enc || !err) return PLBM_ERR_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    {   // rows of 128 pixels: the halo-row kernel where its accumulators fit the TMEM
        const int kbx = Cin / TC_KB, gch = (Cout + TC_KB - 1) / TC_KB;
        const int hstage = 3 * kbx * HALO_ROW_BYTES + gch * WG_CHUNK;
        const int hbudget = 227 * 1024 - WG_SLACK - 1024 - 256;
        const int hst = hbudget / hstage < 4 ? hbudget / hstage : 4;
        if (W % TC_BM == 0 && 3 * kbx * gch * TC_KB <= 512 && hst >= 2) {
            WhArgs h{};
            h.gw = gw; h.g = (const __nv_bfloat16 *)g;
            h.N = N; h.H = H; h.W = W; h.Cin = Cin; h.Cout = Cout;
            h.tiles_x = W / TC_BM; h.total_tiles = N * H * h.tiles_x;
            h.kbx = kbx; h.gchunks = gch; h.stage_bytes = hstage; h.stages = hst;
            h.g_tma = Cout % TC_KB == 0;
            h.err = err;
            h.tiles_per_cta = (h.total_tiles + sms - 1) / sms;
            const int smem = hst * hstage + WG_SLACK + 1024 + 256;
            static int hattr = 0;
            static std::mutex hmu;
            {
                std::lock_guard<std::mutex> lk(hmu);
                if (smem > hattr) {
                    if (cudaFuncSetAttribute(k_wgrad_halo_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
                        return PLBM_ERR_CUDA;
                    hattr = smem;
                }
            }
            CUtensorMap hmap, gmap;
            memset(&gmap, 0, sizeof(gmap));
            const cuuint32_t es[4] = { 1, 1, 1, 1 };
            {
                const cuuint64_t dims[4] = { (cuuint64_t)Cin, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N };
                const cuuint64_t strides[3] = { (cuuint64_t)Cin * 2, (cuuint64_t)W * Cin * 2, (cuuint64_t)H * W * Cin * 2 };
                const cuuint32_t box[4] = { TC_KB, HALO_ROW, 1, 1 };
                if (enc(&hmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(x), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
                    return PLBM_ERR_ARGUMENT;
            }
            if (h.g_tma) {
                const cuuint64_t dims[4] = { (cuuint64_t)Cout, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N };
                const cuuint64_t strides[3] = { (cuuint64_t)Cout * 2, (cuuint64_t)W * Cout * 2, (cuuint64_t)H * W * Cout * 2 };
                const cuuint32_t box[4] = { TC_KB, TC_BM, 1, 1 };
                if (enc(&gmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(g), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
                    return PLBM_ERR_ARGUMENT;
            }
            k_wgrad_halo_tc<<<(h.total_tiles + h.tiles_per_cta - 1) / h.tiles_per_cta, 128, smem, s>>>(hmap, gmap, h);
            return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
        }
    }
    WgArgs a{};
    a.gw = gw; a.g = (const __nv_bfloat16 *)g;
    a.N = N; a.H = H; a.W = W; a.Cin = Cin; a.Cout = Cout;
    a.BW = W >= TC_BM ? TC_BM : W; a.BH = TC_BM / a.BW; a.tiles_x = W / a.BW; a.tiles_y = H / a.BH;
    const int kbx = Cin / TC_KB;
    a.ntaps = kbx == 1 ? 9 : 3;                    // the TMEM columns of a CTA stay <= 384
    a.tg = a.ntaps * kbx <= 9 ? a.ntaps : 1;       // at most nine input tiles (72 KB) per stage
    a.xchunks = a.tg * kbx;
    a.gchunks = (Cout + TC_KB - 1) / TC_KB;
    a.g_tma = Cout % TC_KB == 0;
    // one CTA per SM with 2-4 stages (two CTAs of one stage each measured slower: each then waits
    // out its own load latency)
    const int budget = 227 * 1024 - WG_SLACK - 1024 - 256;
    a.gb = gb;
    a.ones = gb && a.xchunks % 4 != 0 && budget / ((a.xchunks + 1 + a.gchunks) * WG_CHUNK) >= 2 ? 1 : 0;
    a.stage_bytes = (a.xchunks + a.ones + a.gchunks) * WG_CHUNK;
    a.stages = budget / a.stage_bytes < 4 ? budget / a.stage_bytes : 4;
    if (a.stages < 2) return PLBM_ERR_ARGUMENT;
    a.err = err;
    const int smem = a.stages * a.stage_bytes + WG_SLACK + 1024 + 256;
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
    memset(&gmap, 0, sizeof(gmap));
    const cuuint32_t es[4] = { 1, 1, 1, 1 };
    for (int which = 0; which < (a.g_tma ? 2 : 1); ++which) {
        const int C = which == 0 ? Cin : Cout;
        const cuuint64_t dims[4] = { (cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N };
        const cuuint64_t strides[3] = { (cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2 };
        const cuuint32_t box[4] = { TC_KB, (cuuint32_t)a.BW, (cuuint32_t)a.BH, 1 };
        if (enc(which == 0 ? &xmap : &gmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(which == 0 ? x : g),
                dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return PLBM_ERR_ARGUMENT;
    }
    const int groups = 9 / a.ntaps;
    a.total_tiles = N * a.tiles_x * a.tiles_y;
    // one CTA per SM (the stages fill its shared memory): groups x chunks must not exceed the SMs,
    // or the CTAs past them run as a second wave
    const int chunks = sms / groups > 0 ? sms / groups : 1;
    a.tiles_per_cta = (a.total_tiles + chunks - 1) / chunks;
    k_wgrad_tc<<<dim3((a.total_tiles + a.tiles_per_cta - 1) / a.tiles_per_cta, groups), 128, smem, s>>>(xmap, gmap, a);
    if (cudaGetLastError() != cudaSuccess) return PLBM_ERR_CUDA;
    if (bias_done) *bias_done = a.ones;
    return PLBM_OK;
}

// Forward convolution of a narrow input (9 * Cin <= 64, Cout <= 64: eight CTAs of at most 64 TMEM
// columns share an SM) with the im2col tile written by the CTA's threads.
bool plbm_nn_tc_small_supported(int H, int W, int Cin, int Cout)
{
    if (Cin < 1 || 9 * Cin > 2 * TC_KB || Cout < 1 || Cout > 64) return false;
    return tiles_exactly(H, W);
}

int plbm_nn_tc_small_conv(const void *x, const void *w, const float *bias, void *y, int N, int H, int W, int Cin,
                          int Cout, int relu, cudaStream_t s)
{
    int *err = error_flag();
    if (!err) return PLBM_ERR_CUDA;
    SmallArgs a{};
    a.x = (const __nv_bfloat16 *)x; a.w = (const __nv_bfloat16 *)w; a.bias = bias; a.y = (__nv_bfloat16 *)y;
    a.N = N; a.H = H; a.W = W; a.Cin = Cin; a.Cout = Cout; a.npad = (Cout + 15) / 16 * 16; a.relu = relu;
    a.BW = W >= TC_BM ? TC_BM : W; a.BH = TC_BM / a.BW; a.tiles_x = W / a.BW; a.tiles_y = H / a.BH;
    a.kchunks = (9 * Cin + TC_KB - 1) / TC_KB;
    a.err = err;
    const int smem = a.kchunks * (WG_CHUNK + a.npad * 64) + 1024 + 64;
    k_conv_small_tc<<<N * a.tiles_x * a.tiles_y, SM_BUILD, smem, s>>>(a);
    return cudaGetLastError() == cudaSuccess ? PLBM_OK : PLBM_ERR_CUDA;
}

// Weight gradient of a layer with Cin <= 32 (its 9 * Cin (tap, ci) columns in at most 9 chunks of 32)
// and Cout <= 128, both operands written by the CTA's threads.
bool plbm_nn_tc_small_wgrad_supported(int H, int W, int Cin, int Cout)
{
    if (Cin < 1 || Cin > TC_KB || Cout < 1 || Cout > WG_M) return false;
    return tiles_exactly(H, W);
}

int plbm_nn_tc_small_wgrad(const void *x, const void *g, float *gw, int N, int H, int W, int Cin, int Cout,
                           cudaStream_t s)
{
    int *err = error_flag();
    if (!err) return PLBM_ERR_CUDA;
    SmallArgs a{};
    a.x = (const __nv_bfloat16 *)x; a.g = (const __nv_bfloat16 *)g; a.gw = gw;
    a.N = N; a.H = H; a.W = W; a.Cin = Cin; a.Cout = Cout;
    a.BW = W >= TC_BM ? TC_BM : W; a.BH = TC_BM / a.BW; a.tiles_x = W / a.BW; a.tiles_y = H / a.BH;
    a.bchunks = (9 * Cin + TC_KB - 1) / TC_KB;
    a.stage_bytes = (a.bchunks > 4 ? a.bchunks : 4) * WG_CHUNK + (Cout + TC_KB - 1) / TC_KB * WG_CHUNK;
    a.err = err;
    const int smem = 2 * a.stage_bytes + WG_SLACK + 1024 + 64;
    static int attr_bytes = 0;
    static std::mutex mu;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (smem > attr_bytes) {
            if (cudaFuncSetAttribute(k_wgrad_small_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
                return PLBM_ERR_CUDA;
            attr_bytes = smem;
        }
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    a.total_tiles = N * a.tiles_x * a.tiles_y;
    // two CTAs per SM (two MMA issuers, one building while the other's MMAs run) where they fit
    const int per_sm = 2 * smem <= 227 * 1024 ? 2 : 1;
    a.tiles_per_cta = (a.total_tiles + per_sm * sms - 1) / (per_sm * sms);
    k_wgrad_small_tc<<<(a.total_tiles + a.tiles_per_cta - 1) / a.tiles_per_cta, WS_THREADS, smem, s>>>(a);
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
    return plbm_nn_tc_supported(H, W, Cin, Cout) || plbm_nn_tc_small_supported(H, W, Cin, Cout) ? 1 : 0;
}

extern "C" int plbm_nn_wgrad_on_tensor_cores(int H, int W, int Cin, int Cout)
{
    return plbm_nn_tc_wgrad_supported(H, W, Cin, Cout) || plbm_nn_tc_small_wgrad_supported(H, W, Cin, Cout) ? 1 : 0;
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
