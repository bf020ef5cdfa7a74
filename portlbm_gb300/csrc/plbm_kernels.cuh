// plbm_kernels.cuh — the fused per-timestep kernels.  One launch performs what the reference
// does with EmplaceBounceBackKernel + OutletUpdateKernel + StreamCollideKernel (+ buffer
// refreshes for the one-lattice algorithms): every fluid node gathers its nine incoming
// populations (bounce-back and boundary values resolved at the gather), collides, and writes
// its nine outgoing populations once.
//
//   nptl  two lattices, 2-D thread blocks over the inner grid            (nptl.hpp:56-141)
//   lptl  two lattices, 1-D launch over the linear node index            (lptl.hpp:57-137)
//   npol  one lattice, updated in place tile by tile; values crossing a tile edge are read
//         from a double-buffered halo snapshot written by the neighbouring tile in the previous
//         step (replaces the buffer rows/columns and their copy kernels, buffered.hpp:44-153)
//   nsol  one lattice, in-place "AA" swap: even steps read the neighbours' opposite slots and
//         write into the neighbours' slots, odd steps read and write the node's own slots, so
//         every slot is read and written by one thread only (replaces the local-memory swap,
//         nsol_kernels.hpp:171-334)
#pragma once

#include "plbm_device.cuh"
#include "plbm_launch.h"

namespace plbm {

template <int PREC> using CT = typename Store<PREC>::C;

// Incoming population d of inner node (xi, yi) for the pull schemes: ghost constant, own
// opposite value when the source is solid, otherwise the source node's value.
template <int PREC, int L>
__device__ __forceinline__ CT<PREC> pull_one(const void *S, unsigned long long n, int xi, int yi, int d,
                                             uint16_t links, const StepParams &p)
{
    const int sx = xi - cxd(d), sy = yi - cyd(d);
    if (sx < 0 || sx >= p.W || sy < 0 || sy >= p.H) {
        if (sy < 0 || sy >= p.H) {
            if constexpr (shifted<PREC>()) return p.weightf[d] + p.shift_wg[d] * (float)xi;   // w_d (1 - rho0(x'))
            else return g_weight<PREC>(p, d);
        }
        return sx < 0 ? g_in<PREC>(p, d) : g_out<PREC>(p, d);
    }
    if (links & (1u << d)) return ld<PREC>(S, lidx<L>(n, 8 - d, p.N), 8 - d, p);
    const unsigned long long s = (unsigned long long)sx + (unsigned long long)sy * p.P;
    if constexpr (shifted<PREC>()) {
        if (cxd(d) != 0) return ld<PREC>(S, lidx<L>(s, d, p.N), d, p) + p.shift_cx[d];
    }
    return ld<PREC>(S, lidx<L>(s, d, p.N), d, p);
}

// Index offset from node n's entry of direction k to node (n + dn)'s entry of direction k, where
// dn = -cx_d - cy_d * P is the pull source of direction d.
template <int L>
__device__ __forceinline__ long long pull_delta(int d, const StepParams &p)
{
    const long long dn = -(long long)cxd(d) - (long long)cyd(d) * p.P;
    return L == COLLISION ? 9 * dn : (L == STREAM ? dn : 3 * dn);
}

// The float forms write their observables through a separate (not inlined) function taking the
// four moments by value, so its FP64 widening is never scheduled into the per-node path (GB300
// issues FP64 at 1/64 of the FP32 rate); the other forms write inline.
template <int PREC>
__device__ __noinline__ void observables_out(MomentsF m, int x, int y, const StepParams &p)
{
    observables<PREC>(m, x, y, p);
}

template <int PREC>
__device__ __forceinline__ void emit_observables(const MomentsOf<PREC> &m, int x, int y, const StepParams &p)
{
    if constexpr (sizeof(typename Store<PREC>::C) == 4) {
        if (p.write_results || x == p.W - 2) observables_out<PREC>(m, x, y, p);
    } else {
        observables<PREC>(m, x, y, p);
    }
}

// Launch bounds of the nptl, lptl and npol step kernels: the Q60 form runs 256-thread blocks and
// is limited by memory latency, so it is held to 48 registers for a fifth resident block per SM
// (measured faster despite a few spilled words; nsol measured equal and keeps its registers).
template <int PREC> struct NptlBounds { static constexpr int threads = 512, blocks = 1; };
template <> struct NptlBounds<F64_Q60> { static constexpr int threads = 256, blocks = 5; };

// Collision (AoS) layout: the 32 nodes of a warp that lies in one row (or one run of the linear
// index) own 32 consecutive records, 288 consecutive entries of the destination lattice.  Written
// one direction at a time, a warp's 8-byte stores sit 72 bytes apart and touch 32 sectors each; when
// every lane holds a fluid node the warp instead stages its records in a shared-memory slice of its
// own (one __syncwarp, no block barrier) and writes the 288 entries as nine contiguous 32-lane stores
// (8 sectors each).  Warps with a solid or padding lane keep the direct stores, so nodes that are
// not fluid are never written, as before.
template <int PREC> __host__ __device__ constexpr int stage_warps() { return NptlBounds<PREC>::threads / 32; }

template <int PREC>
__device__ __forceinline__ typename Store<PREC>::T encode_value(typename Store<PREC>::C v, const StepParams &p)
{
    if constexpr (PREC == F16S) return __float2half_rn(v);
    else if constexpr (PREC == BF16S) return __float2bfloat16_rn(v);
    else if constexpr (PREC == F16C) {
        bool over;
        const unsigned short b = (unsigned short)f16c_bits(v, over);
        if (over) atomicOr(p.status, 1);
        return b;
    } else return v;
}

// dst: the lattice written; REVERSED writes value d into slot 8 - d (nsol's odd step).
template <int PREC, bool REVERSED = false>
__device__ __forceinline__ void store_records_staged(const StepParams &p, void *dst_lattice, unsigned long long n,
                                                     const CT<PREC> f[9], bool fluid)
{
    using T = typename Store<PREC>::T;
    __shared__ T stage[stage_warps<PREC>()][9 * 32];
    const unsigned lane = threadIdx.x & 31u;
    const unsigned warp = (threadIdx.y * blockDim.x + threadIdx.x) >> 5;
    if (__ballot_sync(0xffffffffu, fluid) != 0xffffffffu) {
        if (fluid) {
#pragma unroll
            for (int d = 0; d < 9; ++d) {
                const int k = REVERSED ? 8 - d : d;
                st<PREC>(dst_lattice, 9ull * n + k, k, f[d], p);
            }
        }
        return;
    }
    T *slice = stage[warp];
#pragma unroll
    for (int d = 0; d < 9; ++d) slice[lane * 9 + (REVERSED ? 8 - d : d)] = encode_value<PREC>(f[d], p);
    __syncwarp();
    const unsigned long long first = 9ull * (n - lane);   // the record of the warp's first node
    T *dst = static_cast<T *>(dst_lattice) + first;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        if (in_range(first + 32u * k + lane, p.lat_elems, p)) dst[32u * k + lane] = slice[32u * k + lane];
    }
    __syncwarp();
}

// Rows per thread: a node of the 2-byte forms moves only 36 B, so each thread issues the loads of
// several nodes before computing any of them to keep enough bytes in flight per SM.
template <int PREC> struct RowsPerThread { static constexpr int value = rows_per_thread(PREC); };

// The gather of one node.  Away from the domain edge every source is the neighbour or, behind a
// solid, the node's own opposite population (pull_one); edge nodes take pull_one.  Three forms,
// chosen by measurement, give the same values:
//  * unshifted storage: interior nodes without solid neighbours load plainly, nodes next to an
//    obstacle select each source; no loaded value is used inside the branches, so a warp split
//    between them waits for one round of loads;
//  * shifted storage, POROUS: one selected load per direction for every interior node, the
//    re-referencing shift added after the branches (domains full of obstacles);
//  * shifted storage otherwise: plain loads and the shift for interior nodes without solid
//    neighbours, pull_one for the rest (open channels).
// STAGED (collision layout, NY == 1, called by whole warps whose 32 nodes are consecutive):
// the destination records are written through store_records_staged.
template <int PREC, int L, int NY, bool POROUS = false, bool STAGED = false>
__device__ __forceinline__ void update_two_lattice_rows(const int xi[NY], const int yi[NY], const StepParams &p)
{
    static_assert(!STAGED || (L == COLLISION && NY == 1), "staged stores: collision layout, one node per thread");
    constexpr bool SH = shifted<PREC>();
    CT<PREC> f[NY][9];
    uint16_t lk[NY];
    unsigned long long n[NY];
#pragma unroll
    for (int j = 0; j < NY; ++j) {
        const bool in = xi[j] < p.W && yi[j] < p.H;
        n[j] = in ? (unsigned long long)xi[j] + (unsigned long long)yi[j] * p.P : 0;
        lk[j] = in ? link_at(p, n[j]) : 0;
    }
#pragma unroll
    for (int j = 0; j < NY; ++j) {
        const bool interior = (lk[j] & (LINK_FLUID | LINK_EDGE)) == LINK_FLUID;
        if ((!SH || !POROUS) && lk[j] == LINK_FLUID) {
#pragma unroll
            for (int d = 0; d < 9; ++d) {
                f[j][d] = ld<PREC>(p.lat0, lidx<L>(n[j], d, p.N) + pull_delta<L>(d, p), d, p);
                if constexpr (SH && !POROUS)
                    if (cxd(d) != 0) f[j][d] += p.shift_cx[d];
            }
        } else if ((!SH || POROUS) && interior) {
#pragma unroll
            for (int d = 0; d < 9; ++d) {
                const bool bounce = d != 4 && ((lk[j] >> d) & 1u);
                f[j][d] = ld<PREC>(p.lat0, bounce ? lidx<L>(n[j], 8 - d, p.N) : lidx<L>(n[j], d, p.N) + pull_delta<L>(d, p),
                                   d, p);
            }
        } else if (lk[j] & LINK_FLUID) {
#pragma unroll
            for (int d = 0; d < 9; ++d) f[j][d] = pull_one<PREC, L>(p.lat0, n[j], xi[j], yi[j], d, lk[j], p);
        }
    }
    if constexpr (STAGED) {
        const bool fluid = (lk[0] & LINK_FLUID) != 0;
        MomentsOf<PREC> m{};
        if (fluid) {
            if constexpr (SH && POROUS) {
                if (!(lk[0] & LINK_EDGE)) {
#pragma unroll
                    for (int d = 0; d < 9; ++d)
                        if (cxd(d) != 0 && !((lk[0] >> d) & 1u)) f[0][d] += p.shift_cx[d];
                }
            }
            if (is_outlet_row(xi[0], yi[0], p)) outlet_fill<PREC>(f[0], jy_prev_at(p, yi[0]), p);
            m = collide<PREC>(f[0], p);
        }
        store_records_staged<PREC>(p, p.lat1, n[0], f[0], fluid);
        if (fluid) emit_observables<PREC>(m, xi[0], yi[0], p);
    } else {
#pragma unroll
        for (int j = 0; j < NY; ++j) {
            if (!(lk[j] & LINK_FLUID)) continue;
            if constexpr (SH && POROUS) {
                // values pulled from the neighbouring columns are re-referenced to this node's rho0
                if (!(lk[j] & LINK_EDGE)) {
#pragma unroll
                    for (int d = 0; d < 9; ++d)
                        if (cxd(d) != 0 && !((lk[j] >> d) & 1u)) f[j][d] += p.shift_cx[d];
                }
            }
            if (is_outlet_row(xi[j], yi[j], p)) outlet_fill<PREC>(f[j], jy_prev_at(p, yi[j]), p);
            const auto m = collide<PREC>(f[j], p);
#pragma unroll
            for (int d = 0; d < 9; ++d) st<PREC>(p.lat1, lidx<L>(n[j], d, p.N), d, f[j][d], p);
            emit_observables<PREC>(m, xi[j], yi[j], p);
        }
    }
}

// nptl: 2-D blocks (tile shape from the work-group size hint); each thread updates NY
// consecutive rows of its column.

template <int PREC, int L, bool POROUS = false>
__global__ void __launch_bounds__(NptlBounds<PREC>::threads, NptlBounds<PREC>::blocks) k_nptl(StepParams p)
{
    constexpr int NY = RowsPerThread<PREC>::value;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y0 = (blockIdx.y * blockDim.y + threadIdx.y) * NY;
    if constexpr (L == COLLISION && NY == 1) {
        if ((blockDim.x & 31u) == 0) {
            // whole warps lie in one row: leave (warp-uniformly) only past the last row or the
            // padded row; lanes past W take part in the staged store as non-fluid nodes
            if (y0 >= p.H || x - (int)(threadIdx.x & 31u) >= p.P) return;
            const int xs[1] = { x }, ys[1] = { y0 };
            update_two_lattice_rows<PREC, L, 1, POROUS, true>(xs, ys, p);
            return;
        }
    }
    if (x >= p.W || y0 >= p.H) return;
    int xi[NY], yi[NY];
#pragma unroll
    for (int j = 0; j < NY; ++j) { xi[j] = x; yi[j] = y0 + j; }
    update_two_lattice_rows<PREC, L, NY, POROUS>(xi, yi, p);
}

// nptl, stream layout, 2-byte storage (F16S / BF16S): each thread updates VEC consecutive nodes
// of one row with a single 16-byte load and store per population plane; a warp covers 256
// consecutive nodes.  The value a node pulls across its vector's edge (x - 1 or x + 1) comes from
// the neighbouring lane by a warp shuffle, or at the warp's edge from one 2-byte load.  Nodes
// that are not interior fluid re-gather their populations with the scalar pull (bounce-back,
// inlet/outlet and wall ghosts), so the arithmetic and the results are those of k_nptl.  Solid
// nodes and row padding are written back as the rest state (df = 0), which is what they hold.
constexpr int VEC = 8;
constexpr int VEC_ROWS = 4;   // rows (warps) per block

// Two packed 2-byte values <-> two floats with one conversion instruction each way; the same
// values and round-to-nearest-even results as ld<PREC> / st<PREC>.
// `shift` re-references the two values to the reading node's rho0 (shift_cx of the plane).
template <int PREC> __device__ __forceinline__ float2 vec_unpack(unsigned w, float shift)
{
    if constexpr (PREC == F16S) {
        __half2 h = *reinterpret_cast<__half2 *>(&w);
        const float2 v = __half22float2(h);
        return make_float2(v.x + shift, v.y + shift);
    } else if constexpr (PREC == F16C) {
        return make_float2(f16c_value(w & 0xffffu) + shift, f16c_value(w >> 16) + shift);
    } else {
        __nv_bfloat162 h = *reinterpret_cast<__nv_bfloat162 *>(&w);
        const float2 v = __bfloat1622float2(h);
        return make_float2(v.x + shift, v.y + shift);
    }
}
// F16C: a value beyond the format's range sets `over` (the caller reports it once per thread).
template <int PREC> __device__ __forceinline__ unsigned vec_pack(float lo, float hi, bool &over)
{
    if constexpr (PREC == F16S) {
        __half2 h = __floats2half2_rn(lo, hi);
        return *reinterpret_cast<unsigned *>(&h);
    } else if constexpr (PREC == F16C) {
        // f16c_bits for two values, the range test on the OR of both rounded patterns
        const unsigned ba = __float_as_uint(lo * F16C_ENCODE), bb = __float_as_uint(hi * F16C_ENCODE);
        const unsigned ra = f16c_round(ba), rb = f16c_round(bb);
        over |= ((ra | rb) & ~F16C_MAX_BITS) != 0;
        return (ra & F16C_MAX_BITS) | ((ba >> 16) & 0x8000u) | ((rb & F16C_MAX_BITS) << 16) | (bb & 0x80000000u);
    } else {
        __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
        return *reinterpret_cast<unsigned *>(&h);
    }
}

// The scalar gather of a vector-kernel node that is not interior fluid (edges, obstacles, outlet).
template <int PREC>
__device__ __forceinline__ void vec_edge_gather(float *f, int x, int y, uint16_t lk, const StepParams &p)
{
    const unsigned long long n = (unsigned long long)x + (unsigned long long)y * p.P;
#pragma unroll
    for (int d = 0; d < 9; ++d) f[d] = pull_one<PREC, STREAM>(p.lat0, n, x, y, d, lk, p);
    if (is_outlet_row(x, y, p)) outlet_fill<PREC>(f, jy_prev_at(p, y), p);
}

template <int PREC>
__device__ __forceinline__ void vec_node(float f[9], int x, int y, uint16_t lk, bool inner_row, bool live,
                                         const StepParams &p)
{
    if (live) {
        // lk == LINK_FLUID: fluid, every source fluid, off the domain edge (links carry LINK_EDGE)
        if (lk != LINK_FLUID) vec_edge_gather<PREC>(f, x, y, lk, p);
        const MomentsF m = collide<PREC>(f, p);
        emit_observables<PREC>(m, x, y, p);
    } else {
#pragma unroll
        for (int d = 0; d < 9; ++d) f[d] = 0.0f;
    }
}

// One warp updates the row segment of row y whose lane `lane` owns nodes xv .. xv + VEC - 1
// (xv = segment start + VEC * lane; lanes past the row's padding idle).  Called by the whole warp.
template <int PREC>
__device__ __forceinline__ void vec_row_segment(const StepParams &p, int y, int xv, int lane)
{
    static_assert(PREC == F16S || PREC == BF16S || PREC == F16C, "2-byte shifted storage only");
    const bool vec_ok = xv < p.P;
    const int x0 = vec_ok ? xv : p.P - VEC;                    // clamped: every lane loads inside the row
    const unsigned short *S = static_cast<const unsigned short *>(p.lat0);
    const size_t row0 = (size_t)y * p.P;
    const bool inner_row = y > 0 && y < p.H - 1;

    // r[d][k]: plane d's values for nodes x0 + 2k (low half) and x0 + 2k + 1 (high half)
    unsigned r[9][4];
    const uint4 l4 = in_range(row0 + x0 + VEC - 1, p.N, p) ? *reinterpret_cast<const uint4 *>(p.links + row0 + x0)
                                                         : make_uint4(0, 0, 0, 0);
    if (inner_row) {
#pragma unroll
        for (int d = 0; d < 9; ++d) {   // all nine loads are issued before any is used
            const size_t at = (size_t)d * p.N + (size_t)(y - cyd(d)) * p.P + x0;
            const uint4 v = in_range(at + VEC - 1, p.lat_elems, p) ? *reinterpret_cast<const uint4 *>(S + at)
                                                                  : make_uint4(0, 0, 0, 0);
            r[d][0] = v.x; r[d][1] = v.y; r[d][2] = v.z; r[d][3] = v.w;
        }
#pragma unroll
        for (int d = 0; d < 9; ++d) {
            const unsigned short *row = S + (size_t)d * p.N + (size_t)(y - cyd(d)) * p.P;
            if (cxd(d) == 1) {            // source x - 1: shift up by one node, the previous lane's last node in front
                unsigned prev = __shfl_up_sync(0xffffffffu, r[d][3] >> 16, 1);
                if (lane == 0)
                    prev = x0 >= 1 && in_range((size_t)(row - S) + x0 - 1, p.lat_elems, p) ? (unsigned)row[x0 - 1] : 0u;
                r[d][3] = __byte_perm(r[d][2], r[d][3], 0x5432);
                r[d][2] = __byte_perm(r[d][1], r[d][2], 0x5432);
                r[d][1] = __byte_perm(r[d][0], r[d][1], 0x5432);
                r[d][0] = __byte_perm(prev, r[d][0], 0x5410);
            } else if (cxd(d) == -1) {    // source x + 1: shift down by one node, the next lane's first node behind
                unsigned next = __shfl_down_sync(0xffffffffu, r[d][0] & 0xffffu, 1);
                if (lane == 31)
                    next = x0 + VEC < p.P && in_range((size_t)(row - S) + x0 + VEC, p.lat_elems, p) ? (unsigned)row[x0 + VEC]
                                                                                                    : 0u;
                r[d][0] = __byte_perm(r[d][0], r[d][1], 0x5432);
                r[d][1] = __byte_perm(r[d][1], r[d][2], 0x5432);
                r[d][2] = __byte_perm(r[d][2], r[d][3], 0x5432);
                r[d][3] = __byte_perm(r[d][3], next, 0x5432);
            }
        }
    } else {
#pragma unroll
        for (int d = 0; d < 9; ++d) r[d][0] = r[d][1] = r[d][2] = r[d][3] = 0u;
    }
    const unsigned lw[4] = { l4.x, l4.y, l4.z, l4.w };
    bool over = false;
#pragma unroll
    for (int k = 0; k < 4; ++k) {     // one pair of nodes at a time
        float fa[9], fb[9];
#pragma unroll
        for (int d = 0; d < 9; ++d) {
            // interior nodes take the re-referenced values; edge nodes re-gather them below
            // (-0.0f leaves the x-resting planes exactly as the scalar gather reads them)
            const float2 v = vec_unpack<PREC>(r[d][k], cxd(d) != 0 ? p.shift_cx[d] : -0.0f);
            fa[d] = v.x;
            fb[d] = v.y;
        }
        const int xa = x0 + 2 * k, xb = xa + 1;
        const uint16_t la = (uint16_t)(lw[k] & 0xffffu), lb = (uint16_t)(lw[k] >> 16);
        vec_node<PREC>(fa, xa, y, la, inner_row, vec_ok && xa < p.W && (la & LINK_FLUID), p);
        vec_node<PREC>(fb, xb, y, lb, inner_row, vec_ok && xb < p.W && (lb & LINK_FLUID), p);
#pragma unroll
        for (int d = 0; d < 9; ++d) r[d][k] = vec_pack<PREC>(fa[d], fb[d], over);
    }
    if constexpr (PREC == F16C)
        if (over) atomicOr(p.status, 1);
    if (!vec_ok) return;
    unsigned short *D = static_cast<unsigned short *>(p.lat1);
#pragma unroll
    for (int d = 0; d < 9; ++d) {
        const size_t at = (size_t)d * p.N + row0 + x0;
        if (in_range(at + VEC - 1, p.lat_elems, p))
            *reinterpret_cast<uint4 *>(D + at) = make_uint4(r[d][0], r[d][1], r[d][2], r[d][3]);
    }
}

// The row update for domains full of obstacles, without per-node branches away from the domain
// edge.  Besides the nine shifted row loads, a lane loads its own row (y) of the six planes with a
// vertical component when some lane of the warp has a solid source (the two horizontal planes were
// loaded at row y already; their unshifted words are kept).  A population whose source is solid
// bounces back, i.e. is the node's own value of the opposite direction: per direction the words
// are merged under a mask built from the link words (bit d of each 16-bit half), and the
// re-referencing shift is left out for those halves, as pull_one does.  Edge nodes keep the scalar
// gather.  The same values as pull_one, i.e. as the other kernels.
template <int PREC>
__device__ __forceinline__ void vec_row_segment_porous(const StepParams &p, int y, int xv, int lane)
{
    static_assert(PREC == F16S || PREC == BF16S || PREC == F16C, "2-byte shifted storage only");
    const bool vec_ok = xv < p.P;
    const int x0 = vec_ok ? xv : p.P - VEC;
    const unsigned short *S = static_cast<const unsigned short *>(p.lat0);
    const size_t row0 = (size_t)y * p.P;
    const bool inner_row = y > 0 && y < p.H - 1;

    unsigned r[9][4];
    const uint4 l4 = in_range(row0 + x0 + VEC - 1, p.N, p) ? *reinterpret_cast<const uint4 *>(p.links + row0 + x0)
                                                         : make_uint4(0, 0, 0, 0);
    const unsigned lw[4] = { l4.x, l4.y, l4.z, l4.w };
    // bits 0-3 and 5-8 of both halves: a solid source (bit 4 marks fluid)
    const bool bounce_here = ((lw[0] | lw[1] | lw[2] | lw[3]) & 0x01EF01EFu) != 0;
    const bool bounce_warp = __any_sync(0xffffffffu, inner_row && bounce_here);
    if (inner_row) {
        unsigned o[6][4];   // own row of planes 0, 1, 2, 6, 7, 8
#pragma unroll
        for (int d = 0; d < 9; ++d) {
            const size_t at = (size_t)d * p.N + (size_t)(y - cyd(d)) * p.P + x0;
            const uint4 v = in_range(at + VEC - 1, p.lat_elems, p) ? *reinterpret_cast<const uint4 *>(S + at)
                                                                  : make_uint4(0, 0, 0, 0);
            r[d][0] = v.x; r[d][1] = v.y; r[d][2] = v.z; r[d][3] = v.w;
        }
        if (bounce_warp) {
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                const int e = i < 3 ? i : i + 3;
                const size_t at = (size_t)e * p.N + row0 + x0;
                const uint4 v = in_range(at + VEC - 1, p.lat_elems, p) ? *reinterpret_cast<const uint4 *>(S + at)
                                                                      : make_uint4(0, 0, 0, 0);
                o[i][0] = v.x; o[i][1] = v.y; o[i][2] = v.z; o[i][3] = v.w;
            }
        }
        const unsigned own3[4] = { r[3][0], r[3][1], r[3][2], r[3][3] }, own5[4] = { r[5][0], r[5][1], r[5][2], r[5][3] };
#pragma unroll
        for (int d = 0; d < 9; ++d) {
            const unsigned short *row = S + (size_t)d * p.N + (size_t)(y - cyd(d)) * p.P;
            if (cxd(d) == 1) {
                unsigned prev = __shfl_up_sync(0xffffffffu, r[d][3] >> 16, 1);
                if (lane == 0)
                    prev = x0 >= 1 && in_range((size_t)(row - S) + x0 - 1, p.lat_elems, p) ? (unsigned)row[x0 - 1] : 0u;
                r[d][3] = __byte_perm(r[d][2], r[d][3], 0x5432);
                r[d][2] = __byte_perm(r[d][1], r[d][2], 0x5432);
                r[d][1] = __byte_perm(r[d][0], r[d][1], 0x5432);
                r[d][0] = __byte_perm(prev, r[d][0], 0x5410);
            } else if (cxd(d) == -1) {
                unsigned next = __shfl_down_sync(0xffffffffu, r[d][0] & 0xffffu, 1);
                if (lane == 31)
                    next = x0 + VEC < p.P && in_range((size_t)(row - S) + x0 + VEC, p.lat_elems, p) ? (unsigned)row[x0 + VEC]
                                                                                                    : 0u;
                r[d][0] = __byte_perm(r[d][0], r[d][1], 0x5432);
                r[d][1] = __byte_perm(r[d][1], r[d][2], 0x5432);
                r[d][2] = __byte_perm(r[d][2], r[d][3], 0x5432);
                r[d][3] = __byte_perm(r[d][3], next, 0x5432);
            }
        }
        if (bounce_warp) {
#pragma unroll
            for (int d = 0; d < 9; ++d) {
                if (d == 4) continue;
                const int e = 8 - d;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const unsigned own = e == 3 ? own3[k] : e == 5 ? own5[k] : o[e < 3 ? e : e - 3][k];
                    const unsigned sel = ((lw[k] >> d) & 0x00010001u) * 0xFFFFu;
                    r[d][k] = (r[d][k] & ~sel) | (own & sel);
                }
            }
        }
    } else {
#pragma unroll
        for (int d = 0; d < 9; ++d) r[d][0] = r[d][1] = r[d][2] = r[d][3] = 0u;
    }
    bool over = false;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float fa[9], fb[9];
        const uint16_t la = (uint16_t)(lw[k] & 0xffffu), lb = (uint16_t)(lw[k] >> 16);
#pragma unroll
        for (int d = 0; d < 9; ++d) {
            // re-referenced unless bounced (-0.0f leaves a value exactly as loaded)
            const float sh = cxd(d) != 0 ? p.shift_cx[d] : -0.0f;
            const float2 v = vec_unpack<PREC>(r[d][k], -0.0f);
            fa[d] = v.x + (((la >> d) & 1u) ? -0.0f : sh);
            fb[d] = v.y + (((lb >> d) & 1u) ? -0.0f : sh);
        }
        const int xa = x0 + 2 * k, xb = xa + 1;
        const bool live_a = vec_ok && xa < p.W && (la & LINK_FLUID), live_b = vec_ok && xb < p.W && (lb & LINK_FLUID);
        if (live_a && (la & LINK_EDGE)) vec_edge_gather<PREC>(fa, xa, y, la, p);
        if (live_b && (lb & LINK_EDGE)) vec_edge_gather<PREC>(fb, xb, y, lb, p);
        if (live_a) {
            const MomentsF m = collide<PREC>(fa, p);
            emit_observables<PREC>(m, xa, y, p);
        } else {
#pragma unroll
            for (int d = 0; d < 9; ++d) fa[d] = 0.0f;
        }
        if (live_b) {
            const MomentsF m = collide<PREC>(fb, p);
            emit_observables<PREC>(m, xb, y, p);
        } else {
#pragma unroll
            for (int d = 0; d < 9; ++d) fb[d] = 0.0f;
        }
#pragma unroll
        for (int d = 0; d < 9; ++d) r[d][k] = vec_pack<PREC>(fa[d], fb[d], over);
    }
    if constexpr (PREC == F16C)
        if (over) atomicOr(p.status, 1);
    if (!vec_ok) return;
    unsigned short *D = static_cast<unsigned short *>(p.lat1);
#pragma unroll
    for (int d = 0; d < 9; ++d) {
        const size_t at = (size_t)d * p.N + row0 + x0;
        if (in_range(at + VEC - 1, p.lat_elems, p))
            *reinterpret_cast<uint4 *>(D + at) = make_uint4(r[d][0], r[d][1], r[d][2], r[d][3]);
    }
}

template <int PREC>
__global__ void __launch_bounds__(32 * VEC_ROWS, 4) k_nptl_vec_porous(StepParams p)
{
    const int lane = threadIdx.x;                              // blockDim.x == 32: a warp is a row segment
    const int y = blockIdx.y * VEC_ROWS + threadIdx.y;
    if (y >= p.H) return;                                      // uniform over the warp
    vec_row_segment_porous<PREC>(p, y, (blockIdx.x * 32 + lane) * VEC, lane);
}

template <int PREC>
__global__ void __launch_bounds__(32 * VEC_ROWS, 4) k_nptl_vec(StepParams p)
{
    const int lane = threadIdx.x;                              // blockDim.x == 32: a warp is a row segment
    const int y = blockIdx.y * VEC_ROWS + threadIdx.y;
    if (y >= p.H) return;                                      // uniform over the warp
    vec_row_segment<PREC>(p, y, (blockIdx.x * 32 + lane) * VEC, lane);
}

// lptl: 1-D launch over n = x' + y' * P (padding columns x' >= W idle); each thread updates NY
// nodes one grid-width apart.
template <int PREC, int L, bool POROUS = false>
__global__ void __launch_bounds__(NptlBounds<PREC>::threads, NptlBounds<PREC>::blocks) k_lptl(StepParams p)
{
    constexpr int NY = RowsPerThread<PREC>::value;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    const unsigned long long n0 = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    int xi[NY], yi[NY];
#pragma unroll
    for (int j = 0; j < NY; ++j) {
        const unsigned long long n = n0 + j * stride;
        if (n < p.N) {
            yi[j] = (int)(n / (unsigned)p.P);
            xi[j] = (int)(n - (unsigned long long)yi[j] * p.P);
        } else {
            yi[j] = p.H;
            xi[j] = p.W;
        }
    }
    if constexpr (L == COLLISION && NY == 1) {
        // blockDim.x is a multiple of 32: every warp covers 32 consecutive linear indices
        update_two_lattice_rows<PREC, L, 1, POROUS, true>(xi, yi, p);
        return;
    }
    update_two_lattice_rows<PREC, L, NY, POROUS>(xi, yi, p);
}

// ---- npol: in place, one tile per thread block --------------------------------------------

// Halo snapshot layout (storage type T), structure of arrays: columns first, then rows; one
// contiguous line per (tile boundary b, slot k), so the lanes of a warp along a tile edge read and
// write consecutive entries.
//   col[b][0..2][y'] = dirs 2,5,8 of node (x' = (b+1)*TW - 1, y')   right edge of tile column b
//   col[b][3..5][y'] = dirs 0,3,6 of node (x' = (b+1)*TW,     y')   left edge of tile column b+1
//   row[b][0..2][x'] = dirs 6,7,8 of node (x', y' = (b+1)*TH - 1)   top edge of tile row b
//   row[b][3..5][x'] = dirs 0,1,2 of node (x', y' = (b+1)*TH)       bottom edge of tile row b+1
__device__ __forceinline__ unsigned long long halo_col(const StepParams &p, int b, int y, int k)
{
    return ((unsigned long long)b * 6 + k) * p.H + y;
}
__device__ __forceinline__ unsigned long long halo_row(const StepParams &p, int b, int x, int k)
{
    return (unsigned long long)p.n_col_bounds * p.H * 6 + ((unsigned long long)b * 6 + k) * p.W + x;
}

template <int PREC, int L>
__global__ void __launch_bounds__(NptlBounds<PREC>::threads, NptlBounds<PREC>::blocks) k_npol(StepParams p)
{
    const int TW = p.tile_w, TH = p.tile_h;
    const int tcx = blockIdx.x, tcy = blockIdx.y;
    const int xi = tcx * TW + threadIdx.x, yi = tcy * TH + threadIdx.y;
    const bool inside = xi < p.W && yi < p.H;
    const unsigned long long n = inside ? (unsigned long long)xi + (unsigned long long)yi * p.P : 0;
    const uint16_t lk = inside ? link_at(p, n) : 0;
    const bool fluid = (lk & LINK_FLUID) != 0;
    const int lx = threadIdx.x, ly = threadIdx.y;
    CT<PREC> f[9];
    if (fluid) {
        if (lk == LINK_FLUID) {
            // away from the domain edge, all sources fluid: each source is in the tile, in the
            // left/right neighbour's column snapshot or in the upper/lower neighbour's row snapshot.
            // The choice is a select per direction, so the lanes on a tile edge (two in every warp
            // of a 32-wide tile) run the same instructions as the others instead of a second,
            // divergent pass.  A tile-edge lane here is never on the domain edge, so the
            // neighbouring tile it selects exists; the index of an unselected branch is unused.
#pragma unroll
            for (int d = 0; d < 9; ++d) {
                const int cx = cxd(d), cy = cyd(d);
                const bool col = (cx == 1 && lx == 0) || (cx == -1 && lx == TW - 1);
                const bool row = !col && ((cy == 1 && ly == 0) || (cy == -1 && ly == TH - 1));
                unsigned long long i = lidx<L>(n, d, p.N) + pull_delta<L>(d, p);
                if (cx != 0) {
                    const unsigned long long ic = halo_col(p, cx == 1 ? tcx - 1 : tcx, yi - cy, cx == 1 ? d / 3 : 3 + d / 3);
                    i = col ? ic : i;
                }
                if (cy != 0) {
                    const unsigned long long ir = halo_row(p, cy == 1 ? tcy - 1 : tcy, xi - cx, cy == 1 ? d - 6 : 3 + d);
                    i = row ? ir : i;
                }
                f[d] = ld<PREC>(col || row ? p.halo_in : p.lat0, i, d, p);
            }
        } else {
#pragma unroll
            for (int d = 0; d < 9; ++d) {
                const int cx = cxd(d), cy = cyd(d), sx = xi - cx, sy = yi - cy;
                if (sx < 0 || sx >= p.W || sy < 0 || sy >= p.H || (lk & (1u << d)) || d == 4) {
                    f[d] = pull_one<PREC, L>(p.lat0, n, xi, yi, d, lk, p);
                } else if ((cx == 1 && lx == 0) || (cx == -1 && lx == TW - 1)) {
                    // the source lies in the neighbouring tile column: its boundary snapshot
                    const int k = cx == 1 ? d / 3 : 3 + d / 3;
                    f[d] = ld<PREC>(p.halo_in, halo_col(p, cx == 1 ? tcx - 1 : tcx, sy, k), d, p);
                } else if ((cy == 1 && ly == 0) || (cy == -1 && ly == TH - 1)) {
                    const int k = cy == 1 ? d - 6 : 3 + d;
                    f[d] = ld<PREC>(p.halo_in, halo_row(p, cy == 1 ? tcy - 1 : tcy, sx, k), d, p);
                } else {
                    f[d] = ld<PREC>(p.lat0, lidx<L>(n, d, p.N) + pull_delta<L>(d, p), d, p);
                }
            }
        }
    }
    __syncthreads();   // every read of this tile's old values happens before any write
    // collision layout with whole-warp tile rows: every thread takes part in the staged store
    bool staged = false;
    if constexpr (L == COLLISION) staged = (blockDim.x & 31u) == 0;
    if (!staged && !fluid) return;
    MomentsOf<PREC> m{};
    if (fluid) {
        if (is_outlet_row(xi, yi, p)) outlet_fill<PREC>(f, jy_prev_at(p, yi), p);
        m = collide<PREC>(f, p);
    }
    if (staged) {
        store_records_staged<PREC>(p, p.lat0, n, f, fluid);
        if (!fluid) return;
    } else {
#pragma unroll
        for (int d = 0; d < 9; ++d) st<PREC>(p.lat0, lidx<L>(n, d, p.N), d, f[d], p);
    }
    if (lx == TW - 1 && tcx < p.n_col_bounds)
        for (int k = 0; k < 3; ++k) st<PREC>(p.halo_out, halo_col(p, tcx, yi, k), 3 * k + 2, f[3 * k + 2], p);
    if (lx == 0 && tcx > 0)
        for (int k = 0; k < 3; ++k) st<PREC>(p.halo_out, halo_col(p, tcx - 1, yi, 3 + k), 3 * k, f[3 * k], p);
    if (ly == TH - 1 && tcy < p.n_row_bounds)
        for (int k = 0; k < 3; ++k) st<PREC>(p.halo_out, halo_row(p, tcy, xi, k), 6 + k, f[6 + k], p);
    if (ly == 0 && tcy > 0)
        for (int k = 0; k < 3; ++k) st<PREC>(p.halo_out, halo_row(p, tcy - 1, xi, 3 + k), k, f[k], p);
    emit_observables<PREC>(m, xi, yi, p);
}

// ---- nsol: in-place AA swap ---------------------------------------------------------------
// Slot (m, k) denotes lattice entry lidx(m, k).  Between steps the lattice alternates between
//   state P (before an even step): slot (m, 8-k) holds node m's post-collision value of k;
//   state Q (before an odd step):  slot (m, k) holds the value arriving at m along k.
// The initial rest state is both (weights are symmetric, w_k = w_{8-k}).

// The even-step gather of a fluid node: each source neighbour's reversed slot, the node's own slot
// behind a solid, ghost constants at the domain edge.
template <int PREC, int L>
__device__ __forceinline__ void nsol_even_gather(CT<PREC> f[9], unsigned long long n, int xi, int yi, uint16_t lk,
                                                 const StepParams &p)
{
    if (lk == LINK_FLUID) {   // links carry LINK_EDGE on the domain edge
#pragma unroll
        for (int d = 0; d < 9; ++d) f[d] = ld<PREC>(p.lat0, lidx<L>(n, 8 - d, p.N) + pull_delta<L>(d, p), 8 - d, p);
    } else {
#pragma unroll
        for (int d = 0; d < 9; ++d) {
            const int sx = xi - cxd(d), sy = yi - cyd(d);
            if (d == 4) {
                f[4] = ld<PREC>(p.lat0, lidx<L>(n, 4, p.N), 4, p);
            } else if (sx < 0 || sx >= p.W || sy < 0 || sy >= p.H) {
                f[d] = (sy < 0 || sy >= p.H) ? g_weight<PREC>(p, d) : (sx < 0 ? g_in<PREC>(p, d) : g_out<PREC>(p, d));
            } else if (lk & (1u << d)) {
                f[d] = ld<PREC>(p.lat0, lidx<L>(n, d, p.N), d, p);          // own post-collision 8-d
            } else {
                const unsigned long long s = (unsigned long long)sx + (unsigned long long)sy * p.P;
                f[d] = ld<PREC>(p.lat0, lidx<L>(s, 8 - d, p.N), 8 - d, p);
            }
        }
    }
}

// nsol's even step in the collision (record) layout with its stores staged per block.  A node
// writes value d into slot d of neighbour n + c_d, so written one by one a warp's stores sit 72
// bytes apart and each fills an eighth or a quarter of a sector.  A 32-wide tile of up to
// NSOL_STAGE_ROWS rows has every slot of each of its own records written by its own nodes: the
// block places each new value in a shared-memory copy of the tile's records and their one-node
// frame (with a flag per slot), and after one barrier writes the copy out row by row, consecutive
// threads on consecutive entries, the flagged slots only (the frame's records are shared with the
// neighbouring tiles; slots toward a ghost are never written).  Every slot a node writes is one
// it read itself (the AA pattern), so no other block reads it in this step.
template <int PREC>
__device__ __forceinline__ void nsol_even_collision_staged(const StepParams &p)
{
    using T = typename Store<PREC>::T;
    constexpr int RW = 34, RH = NSOL_STAGE_ROWS + 2, E = RW * 9;   // entries per frame row
    static_assert((RH * E) % 4 == 0, "the flags are cleared as 32-bit words");
    __shared__ T stage[RH * E];
    __shared__ __align__(4) unsigned char written[RH * E];
    const int tid = threadIdx.y * 32 + threadIdx.x, nt = 32 * blockDim.y, rows = blockDim.y + 2;
    // whole words: at most RH * E bytes, since rows <= RH and RH * E is a multiple of four
    for (int i = tid; i < (rows * E + 3) / 4; i += nt) reinterpret_cast<unsigned *>(written)[i] = 0u;
    __syncthreads();
    const int xi = blockIdx.x * 32 + threadIdx.x, yi = blockIdx.y * blockDim.y + threadIdx.y;
    const bool inside = xi < p.W && yi < p.H;
    const unsigned long long n = inside ? (unsigned long long)xi + (unsigned long long)yi * p.P : 0;
    const uint16_t lk = inside ? link_at(p, n) : 0;
    if (lk & LINK_FLUID) {
        CT<PREC> f[9];
        nsol_even_gather<PREC, COLLISION>(f, n, xi, yi, lk, p);
        if (is_outlet_row(xi, yi, p)) outlet_fill<PREC>(f, jy_prev_at(p, yi), p);
        const auto m = collide<PREC>(f, p);
#pragma unroll
        for (int d = 0; d < 9; ++d) {
            const int tx = xi + cxd(d), ty = yi + cyd(d);
            if (tx < 0 || tx >= p.W || ty < 0 || ty >= p.H) continue;   // toward a ghost: never read
            const int i = (threadIdx.y + 1 + cyd(d)) * E + (threadIdx.x + 1 + cxd(d)) * 9 + d;
            stage[i] = encode_value<PREC>(f[d], p);
            written[i] = 1;
        }
        emit_observables<PREC>(m, xi, yi, p);
    }
    __syncthreads();
    // frame row r is lattice row y0 - 1 + r, records x0 - 1 .. x0 + 32: 306 consecutive entries
    const long long x0 = (long long)blockIdx.x * 32, y0 = (long long)blockIdx.y * blockDim.y;
    T *lat = static_cast<T *>(p.lat0);
    for (int i = tid; i < rows * E; i += nt) {
        if (!written[i]) continue;                                      // flagged slots lie in the domain
        const int r = i / E, k = i - r * E;
        const unsigned long long e = 9ull * ((unsigned long long)(y0 - 1 + r) * p.P + (unsigned long long)(x0 - 1)) + k;
        if (in_range(e, p.lat_elems, p)) lat[e] = stage[i];
    }
}

// The staged even step as its own kernel (launched by launch_nsol for 32 x NSOL_STAGE_ROWS blocks
// in the collision layout): 256 threads, four resident blocks (the 64-register cap an unbounded
// kernel gets), five for the Q60 form (48 registers, measured faster).  The other nsol kernels keep
// no launch bounds: a bound above 256 threads let the compiler take 98 registers for the stream
// layout's even step and halved its resident blocks.
template <int PREC>
__global__ void __launch_bounds__(256, PREC == F64_Q60 ? 5 : 4) k_nsol_even_staged(StepParams p)
{
    nsol_even_collision_staged<PREC>(p);
}

template <int PREC, int L>
__global__ void k_nsol_even(StepParams p)
{
    const int xi = blockIdx.x * blockDim.x + threadIdx.x;
    const int yi = blockIdx.y * blockDim.y + threadIdx.y;
    if (xi >= p.W || yi >= p.H) return;
    const unsigned long long n = (unsigned long long)xi + (unsigned long long)yi * p.P;
    const uint16_t lk = link_at(p, n);
    if (!(lk & LINK_FLUID)) return;
    CT<PREC> f[9];
    nsol_even_gather<PREC, L>(f, n, xi, yi, lk, p);
    const bool fast = lk == LINK_FLUID;
    if (is_outlet_row(xi, yi, p)) outlet_fill<PREC>(f, jy_prev_at(p, yi), p);
    const auto m = collide<PREC>(f, p);
    if (fast) {
#pragma unroll
        for (int d = 0; d < 9; ++d) st<PREC>(p.lat0, lidx<L>(n, d, p.N) - pull_delta<L>(d, p), d, f[d], p);
    } else {
#pragma unroll
        for (int d = 0; d < 9; ++d) {
            const int tx = xi + cxd(d), ty = yi + cyd(d);
            if (tx < 0 || tx >= p.W || ty < 0 || ty >= p.H) continue;   // toward a ghost: never read
            const unsigned long long t = (unsigned long long)tx + (unsigned long long)ty * p.P;
            st<PREC>(p.lat0, lidx<L>(t, d, p.N), d, f[d], p);
        }
    }
    emit_observables<PREC>(m, xi, yi, p);
}

// The odd-step gather of a fluid node: its own slots, a bounce-back link's value from the solid
// neighbour's slot, ghost constants at the domain edge.
template <int PREC, int L>
__device__ __forceinline__ void nsol_odd_gather(CT<PREC> f[9], unsigned long long n, int xi, int yi, uint16_t lk,
                                                const StepParams &p)
{
    if (lk == LINK_FLUID) {   // links carry LINK_EDGE on the domain edge
#pragma unroll
        for (int d = 0; d < 9; ++d) f[d] = ld<PREC>(p.lat0, lidx<L>(n, d, p.N), d, p);
    } else {
#pragma unroll
        for (int d = 0; d < 9; ++d) {
            const int sx = xi - cxd(d), sy = yi - cyd(d);
            if (d == 4) {
                f[4] = ld<PREC>(p.lat0, lidx<L>(n, 4, p.N), 4, p);
            } else if (sx < 0 || sx >= p.W || sy < 0 || sy >= p.H) {
                f[d] = (sy < 0 || sy >= p.H) ? g_weight<PREC>(p, d) : (sx < 0 ? g_in<PREC>(p, d) : g_out<PREC>(p, d));
            } else if (lk & (1u << d)) {
                const unsigned long long s = (unsigned long long)sx + (unsigned long long)sy * p.P;
                f[d] = ld<PREC>(p.lat0, lidx<L>(s, 8 - d, p.N), 8 - d, p);  // parked in the solid's slot
            } else {
                f[d] = ld<PREC>(p.lat0, lidx<L>(n, d, p.N), d, p);
            }
        }
    }
}

template <int PREC, int L>
__global__ void k_nsol_odd(StepParams p)
{
    const int xi = blockIdx.x * blockDim.x + threadIdx.x;
    const int yi = blockIdx.y * blockDim.y + threadIdx.y;
    if constexpr (L == COLLISION) {
        // the node's own record, written reversed: whole-warp rows stage it (store_records_staged)
        if ((blockDim.x & 31u) == 0) {
            if (yi >= p.H || xi - (int)(threadIdx.x & 31u) >= p.P) return;   // warp-uniform
            const bool in = xi < p.W;
            const unsigned long long n = in ? (unsigned long long)xi + (unsigned long long)yi * p.P : 0;
            const uint16_t lk = in ? link_at(p, n) : 0;
            const bool fluid = (lk & LINK_FLUID) != 0;
            CT<PREC> f[9];
            MomentsOf<PREC> m{};
            if (fluid) {
                nsol_odd_gather<PREC, L>(f, n, xi, yi, lk, p);
                if (is_outlet_row(xi, yi, p)) outlet_fill<PREC>(f, jy_prev_at(p, yi), p);
                m = collide<PREC>(f, p);
            }
            store_records_staged<PREC, true>(p, p.lat0, n, f, fluid);
            if (fluid) emit_observables<PREC>(m, xi, yi, p);
            return;
        }
    }
    if (xi >= p.W || yi >= p.H) return;
    const unsigned long long n = (unsigned long long)xi + (unsigned long long)yi * p.P;
    const uint16_t lk = link_at(p, n);
    if (!(lk & LINK_FLUID)) return;
    CT<PREC> f[9];
    nsol_odd_gather<PREC, L>(f, n, xi, yi, lk, p);
    if (is_outlet_row(xi, yi, p)) outlet_fill<PREC>(f, jy_prev_at(p, yi), p);
    const auto m = collide<PREC>(f, p);
#pragma unroll
    for (int d = 0; d < 9; ++d) st<PREC>(p.lat0, lidx<L>(n, 8 - d, p.N), 8 - d, f[d], p);
    emit_observables<PREC>(m, xi, yi, p);
}

}  // namespace plbm
