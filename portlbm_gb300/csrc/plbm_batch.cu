// plbm_batch.cu — many independent domains advanced together: one persistent launch per timestep
// walks a queue of tiles drawn from every domain (atomic ticket counter, reset by a memset node),
// and runs of steps are replayed from a captured CUDA graph.  Each domain keeps its own two
// lattices (stream layout), links, geometry, relaxation time and boundary densities; the per-node
// update is the nptl update of plbm_kernels.cuh (FP32, FP16 or BF16 shifted storage, or F64_Q60;
// the 2-byte forms can run the vectorised row update, one warp per 256 consecutive nodes).
//
// There is no counterpart in the reference, which runs one domain per handler.
#include "../../include/plbm_c.h"
#include "plbm_consts.h"
#include "plbm_kernels.cuh"
#include "plbm_launch.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

namespace plbm {

struct BatchArgs {
    const StepParams *params;      // two per domain: parity 0 and 1
    const unsigned *tile_domain;   // domain of each global tile
    const unsigned *tile_local;    // tile index inside its domain
    const int *tiles_x;            // tiles per row of each domain
    unsigned n_tiles;
    unsigned *ticket;              // work-queue counter, zeroed before every step
    int tile_w, tile_h, tile_rows;   // a tile is tile_w x (tile_h * tile_rows) nodes
    unsigned parity;
    int write_results;
};

// Copies one StepParams into shared memory with the whole block, 8 bytes per thread per pass.
__device__ __forceinline__ void stage_params(StepParams &dst, const StepParams &src)
{
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
    unsigned long long *d = reinterpret_cast<unsigned long long *>(&dst);
    const unsigned long long *s = reinterpret_cast<const unsigned long long *>(&src);
    for (int i = tid; i < (int)(sizeof(StepParams) / 8); i += nt) d[i] = s[i];
}

// Persistent: every block takes tiles from the queue until it is empty; the tile's domain
// parameters are staged in shared memory.  The ticket of the next tile is claimed while the
// current one is processed, so the queue's atomic is off the critical path.
template <int PREC>
__global__ void __launch_bounds__(256, PREC == F64_Q60 ? 3 : 6) k_batch(BatchArgs a)
{
    __shared__ __align__(16) StepParams sp;
    __shared__ unsigned s_tile;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    unsigned cur = 0xffffffffu;
    if (tid == 0) s_tile = atomicAdd(a.ticket, 1u);
    __syncthreads();
    for (;;) {
        const unsigned t = s_tile;
        if (t >= a.n_tiles) return;
        const unsigned dom = a.tile_domain[t];
        __syncthreads();   // every thread has read s_tile
        unsigned next = 0;
        if (tid == 0) next = atomicAdd(a.ticket, 1u);
        if (dom != cur) {
            stage_params(sp, a.params[2 * dom + a.parity]);
            __syncthreads();
            if (tid == 0) sp.write_results = a.write_results;
            __syncthreads();
            cur = dom;
        }
        const int local = (int)a.tile_local[t], txs = a.tiles_x[dom];
        const int xi = (local % txs) * a.tile_w + threadIdx.x;
        const int y0 = (local / txs) * a.tile_h * a.tile_rows + threadIdx.y;
        for (int r = 0; r < a.tile_rows; ++r) {
            const int yi = y0 + r * a.tile_h;
            if (xi < sp.W && yi < sp.H) {
                const int xs[1] = { xi }, ys[1] = { yi };
                update_two_lattice_rows<PREC, STREAM, 1, true>(xs, ys, sp);
            }
        }
        if (tid == 0) s_tile = next;
        __syncthreads();   // sp and s_tile are rewritten for the next tile
    }
}

// An inlet or outlet node of an inner row: its row-loaded values are pull_one's for every direction
// whose source lies inside the domain, so only the three directions sourced from the ghost column
// take its constants (x = 0: d = 2, 5, 8 from x = -1; x = W-1: d = 0, 3, 6 from x = W), then the
// outlet refill -- vec_edge_gather's values without its nine scalar loads.
template <int PREC>
__device__ __forceinline__ void vec_edge_column(float *f, int x, int y, const StepParams &p)
{
    if (x == 0) {
        f[2] = g_in<PREC>(p, 2); f[5] = g_in<PREC>(p, 5); f[8] = g_in<PREC>(p, 8);
    }
    if (x == p.W - 1) {
        f[0] = g_out<PREC>(p, 0); f[3] = g_out<PREC>(p, 3); f[6] = g_out<PREC>(p, 6);
    }
    if (is_outlet_row(x, y, p)) outlet_fill<PREC>(f, jy_prev_at(p, y), p);
}

// The porous row update of vec_row_segment_porous with the domain walked in row-major order
// instead of row by row: the lane owns the eight nodes starting at linear node n0 = y * P + x0
// (P, the row pitch, is a multiple of 32, so they lie in one row), and a warp's 256 nodes may span
// rows.  Narrow domains then leave no lanes idle past a row's end.  A lane's neighbour in the warp
// holds the node before (after) its first (last) node whenever that node is in the same row; where
// it is not, the node is on the inlet (outlet) column and the direction sourced across the row end
// is a ghost one, replaced by vec_edge_column.  Every lane takes part in the shuffles; rows 0 and
// H-1 (edge nodes throughout) keep the scalar gather.  The same values as pull_one.
template <int PREC>
__device__ __forceinline__ void vec_linear_segment_porous(const StepParams &p, long long n0, int lane)
{
    const long long nodes = (long long)p.P * p.H;
    const bool vec_ok = n0 < nodes;
    const long long nc = vec_ok ? n0 : nodes - VEC;             // idle lanes load in range
    const int y = (int)(nc / p.P), x0 = (int)(nc - (long long)y * p.P);
    const unsigned short *S = static_cast<const unsigned short *>(p.lat0);
    const bool inner_row = y > 0 && y < p.H - 1;

    const uint4 l4 = in_range(nc + VEC - 1, p.N, p) ? *reinterpret_cast<const uint4 *>(p.links + nc) : make_uint4(0, 0, 0, 0);
    const unsigned lw[4] = { l4.x, l4.y, l4.z, l4.w };
    const bool bounce_here = ((lw[0] | lw[1] | lw[2] | lw[3]) & 0x01EF01EFu) != 0;
    const bool bounce_warp = __any_sync(0xffffffffu, inner_row && bounce_here);
    unsigned r[9][4];
#pragma unroll
    for (int d = 0; d < 9; ++d) {
        const size_t at = (size_t)d * p.N + (size_t)(y - cyd(d)) * p.P + x0;
        const uint4 v = inner_row && in_range(at + VEC - 1, p.lat_elems, p) ? *reinterpret_cast<const uint4 *>(S + at)
                                                                            : make_uint4(0, 0, 0, 0);
        r[d][0] = v.x; r[d][1] = v.y; r[d][2] = v.z; r[d][3] = v.w;
    }
    unsigned o[6][4];   // own row of planes 0, 1, 2, 6, 7, 8
    if (bounce_warp) {
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            const int e = i < 3 ? i : i + 3;
            const size_t at = (size_t)e * p.N + (size_t)nc;
            const uint4 v = inner_row && in_range(at + VEC - 1, p.lat_elems, p) ? *reinterpret_cast<const uint4 *>(S + at)
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
                prev = inner_row && x0 >= 1 && in_range((size_t)(row - S) + x0 - 1, p.lat_elems, p) ? (unsigned)row[x0 - 1] : 0u;
            r[d][3] = __byte_perm(r[d][2], r[d][3], 0x5432);
            r[d][2] = __byte_perm(r[d][1], r[d][2], 0x5432);
            r[d][1] = __byte_perm(r[d][0], r[d][1], 0x5432);
            r[d][0] = __byte_perm(prev, r[d][0], 0x5410);
        } else if (cxd(d) == -1) {
            unsigned next = __shfl_down_sync(0xffffffffu, r[d][0] & 0xffffu, 1);
            if (lane == 31)
                next = inner_row && x0 + VEC < p.P && in_range((size_t)(row - S) + x0 + VEC, p.lat_elems, p)
                           ? (unsigned)row[x0 + VEC] : 0u;
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
    bool over = false;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float fa[9], fb[9];
        const uint16_t la = (uint16_t)(lw[k] & 0xffffu), lb = (uint16_t)(lw[k] >> 16);
#pragma unroll
        for (int d = 0; d < 9; ++d) {
            const float sh = cxd(d) != 0 ? p.shift_cx[d] : -0.0f;
            const float2 v = vec_unpack<PREC>(r[d][k], -0.0f);
            fa[d] = v.x + (((la >> d) & 1u) ? -0.0f : sh);
            fb[d] = v.y + (((lb >> d) & 1u) ? -0.0f : sh);
        }
        const int xa = x0 + 2 * k, xb = xa + 1;
        const bool live_a = vec_ok && xa < p.W && (la & LINK_FLUID), live_b = vec_ok && xb < p.W && (lb & LINK_FLUID);
        if (live_a && (la & LINK_EDGE)) {
            if (inner_row) vec_edge_column<PREC>(fa, xa, y, p);
            else vec_edge_gather<PREC>(fa, xa, y, la, p);
        }
        if (live_b && (lb & LINK_EDGE)) {
            if (inner_row) vec_edge_column<PREC>(fb, xb, y, p);
            else vec_edge_gather<PREC>(fb, xb, y, lb, p);
        }
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
        const size_t at = (size_t)d * p.N + (size_t)nc;
        if (in_range(at + VEC - 1, p.lat_elems, p))
            *reinterpret_cast<uint4 *>(D + at) = make_uint4(r[d][0], r[d][1], r[d][2], r[d][3]);
    }
}

// 2-byte storage: the same queue, each warp updating 256 consecutive nodes of a domain's row-major
// order with the vectorised row update of k_nptl_vec_porous (vec_linear_segment_porous: bounce-back
// merged word-wise, no per-node branches away from the domain edge; blockDim.x == 32; a tile is
// tile_h * tile_rows such segments).  The
// queue loop is repeated rather than shared with k_batch through a tile-body lambda: that version
// compiled k_batch<F32> with more spilled words and ran 1.8 % slower.
template <int PREC>
__global__ void __launch_bounds__(256, 2) k_batch_vec(BatchArgs a)
{
    __shared__ __align__(16) StepParams sp;
    __shared__ unsigned s_tile;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    unsigned cur = 0xffffffffu;
    if (tid == 0) s_tile = atomicAdd(a.ticket, 1u);
    __syncthreads();
    for (;;) {
        const unsigned t = s_tile;
        if (t >= a.n_tiles) return;
        const unsigned dom = a.tile_domain[t];
        __syncthreads();
        unsigned next = 0;
        if (tid == 0) next = atomicAdd(a.ticket, 1u);
        if (dom != cur) {
            stage_params(sp, a.params[2 * dom + a.parity]);
            __syncthreads();
            if (tid == 0) sp.write_results = a.write_results;
            __syncthreads();
            cur = dom;
        }
        // tile `local` is segments local * S .. local * S + S - 1 of the domain's row-major node order
        const long long seg0 = (long long)a.tile_local[t] * (a.tile_h * a.tile_rows) + threadIdx.y;
        const long long nodes = (long long)sp.P * sp.H;
        for (int r = 0; r < a.tile_rows; ++r) {
            const long long base = (seg0 + (long long)r * a.tile_h) * (32 * VEC);
            if (base < nodes) vec_linear_segment_porous<PREC>(sp, base + threadIdx.x * VEC, threadIdx.x);   // warp-uniform
        }
        if (tid == 0) s_tile = next;
        __syncthreads();
    }
}

// One launch per domain with the same per-node update (the comparison the batching form is
// measured against).
template <int PREC>
__global__ void k_batch_single(BatchArgs a, unsigned domain)
{
    __shared__ __align__(16) StepParams sp;
    stage_params(sp, a.params[2 * domain + a.parity]);
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) sp.write_results = a.write_results;
    __syncthreads();
    const int xi = blockIdx.x * blockDim.x + threadIdx.x, yi = blockIdx.y * blockDim.y + threadIdx.y;
    if (xi < sp.W && yi < sp.H) {
        const int xs[1] = { xi }, ys[1] = { yi };
        update_two_lattice_rows<PREC, STREAM, 1, true>(xs, ys, sp);
    }
}

}  // namespace plbm

namespace {

using plbm::StepParams;

}  // namespace

struct plbm_batch {
    int prec = PLBM_F32;
    std::vector<StepParams> host;   // parity 0 and 1 per domain
    std::vector<void *> allocs;
    StepParams *dom_d = nullptr;
    unsigned *tile_domain_d = nullptr, *tile_local_d = nullptr, *ticket_d = nullptr;
    int *tiles_x_d = nullptr;
    int *status_d = nullptr, *status_pending = nullptr;
    unsigned n_tiles = 0, t = 0;
    int tile_w = 32, tile_h = 4, tile_rows = 8, blocks = 0;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t gexec = nullptr;
    unsigned graph_steps = 0;
    std::string err;
    unsigned long long nodes = 0;
    std::vector<unsigned> tile_domain_host;

    ~plbm_batch()
    {
        if (gexec) cudaGraphExecDestroy(gexec);
        for (void *p : allocs) cudaFree(p);
        if (dom_d) cudaFree(dom_d);
        if (tile_domain_d) cudaFree(tile_domain_d);
        if (tile_local_d) cudaFree(tile_local_d);
        if (tiles_x_d) cudaFree(tiles_x_d);
        if (ticket_d) cudaFree(ticket_d);
        if (status_pending) cudaFree(status_pending);
        if (stream) cudaStreamDestroy(stream);
    }

    unsigned n_domains() const { return (unsigned)(host.size() / 2); }
    bool two_byte() const { return prec == PLBM_F16S || prec == PLBM_BF16S || prec == PLBM_F16C; }
    // vectorised rows (2-byte storage only): one warp per 256-node row segment
    bool vec_rows = false;
    bool vec() const { return vec_rows; }
    int tile_nodes_w() const { return vec() ? 32 * plbm::VEC : tile_w; }

    // Tiles of every domain in domain order; the queue hands them out in that order.
    cudaError_t build_tiles()
    {
        std::vector<unsigned> dom, loc;
        std::vector<int> tx;
        for (unsigned i = 0; i < n_domains(); ++i) {
            const StepParams &d = host[2 * i];
            // vectorised rows: tiles of tile_h * tile_rows 256-node segments of the row-major order
            const long long segs = ((long long)d.P * d.H + 32 * plbm::VEC - 1) / (32 * plbm::VEC);
            const int tw = tile_nodes_w();
            const int nx = vec() ? 1 : (d.W + tw - 1) / tw;
            const int ny = vec() ? (int)((segs + tile_h * tile_rows - 1) / (tile_h * tile_rows))
                                 : (d.H + tile_h * tile_rows - 1) / (tile_h * tile_rows);
            tx.push_back(nx);
            for (int k = 0; k < nx * ny; ++k) { dom.push_back(i); loc.push_back((unsigned)k); }
        }
        n_tiles = (unsigned)dom.size();
        // the old arrays may be referenced by the captured graph: drop it first (cudaFree waits for
        // work in flight), and clear each pointer so a failed allocation leaves none dangling
        if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
        if (tile_domain_d) cudaFree(tile_domain_d);
        if (tile_local_d) cudaFree(tile_local_d);
        if (tiles_x_d) cudaFree(tiles_x_d);
        tile_domain_d = tile_local_d = nullptr;
        tiles_x_d = nullptr;
        cudaError_t e = cudaMalloc(&tile_domain_d, n_tiles * sizeof(unsigned));
        if (e == cudaSuccess) e = cudaMalloc(&tile_local_d, n_tiles * sizeof(unsigned));
        if (e == cudaSuccess) e = cudaMalloc(&tiles_x_d, tx.size() * sizeof(int));
        if (e == cudaSuccess) e = cudaMemcpyAsync(tile_domain_d, dom.data(), n_tiles * 4, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(tile_local_d, loc.data(), n_tiles * 4, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(tiles_x_d, tx.data(), tx.size() * 4, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
        return e;
    }

    plbm::BatchArgs args(unsigned parity, int write_results) const
    {
        return plbm::BatchArgs{ dom_d, tile_domain_d, tile_local_d, tiles_x_d, n_tiles, ticket_d,
                                tile_w, tile_h, tile_rows, parity, write_results };
    }

    cudaError_t launch(unsigned step, int write_results)
    {
        cudaError_t e = cudaMemsetAsync(ticket_d, 0, sizeof(unsigned), stream);
        if (e != cudaSuccess) return e;
        const plbm::BatchArgs a = args(step & 1u, write_results);
        const dim3 block(tile_w, tile_h);
        switch (prec) {
        case PLBM_F32: plbm::k_batch<plbm::F32><<<blocks, block, 0, stream>>>(a); break;
        case PLBM_F16S:
            if (vec()) plbm::k_batch_vec<plbm::F16S><<<blocks, block, 0, stream>>>(a);
            else plbm::k_batch<plbm::F16S><<<blocks, block, 0, stream>>>(a);
            break;
        case PLBM_BF16S:
            if (vec()) plbm::k_batch_vec<plbm::BF16S><<<blocks, block, 0, stream>>>(a);
            else plbm::k_batch<plbm::BF16S><<<blocks, block, 0, stream>>>(a);
            break;
        case PLBM_F16C:
            if (vec()) plbm::k_batch_vec<plbm::F16C><<<blocks, block, 0, stream>>>(a);
            else plbm::k_batch<plbm::F16C><<<blocks, block, 0, stream>>>(a);
            break;
        default: plbm::k_batch<plbm::F64_Q60><<<blocks, block, 0, stream>>>(a); break;
        }
        return cudaGetLastError();
    }

    cudaError_t launch_per_domain(unsigned step, int write_results)
    {
        const plbm::BatchArgs a = args(step & 1u, write_results);
        const dim3 block(32, 4);
        for (unsigned i = 0; i < n_domains(); ++i) {
            const dim3 grid((host[2 * i].W + 31) / 32, (host[2 * i].H + 3) / 4);
            switch (prec) {
            case PLBM_F32: plbm::k_batch_single<plbm::F32><<<grid, block, 0, stream>>>(a, i); break;
            case PLBM_F16S: plbm::k_batch_single<plbm::F16S><<<grid, block, 0, stream>>>(a, i); break;
            case PLBM_BF16S: plbm::k_batch_single<plbm::BF16S><<<grid, block, 0, stream>>>(a, i); break;
            case PLBM_F16C: plbm::k_batch_single<plbm::F16C><<<grid, block, 0, stream>>>(a, i); break;
            default: plbm::k_batch_single<plbm::F64_Q60><<<grid, block, 0, stream>>>(a, i); break;
            }
        }
        return cudaGetLastError();
    }

    cudaError_t ensure_graph(unsigned steps_per_graph)
    {
        if (gexec && graph_steps == steps_per_graph) return cudaSuccess;
        if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        cudaError_t el = cudaSuccess;
        for (unsigned k = 0; k < steps_per_graph && el == cudaSuccess; ++k) el = launch(k, 0);
        e = cudaStreamEndCapture(stream, &g);
        if (el != cudaSuccess) return el;
        if (e != cudaSuccess) return e;
        e = cudaGraphInstantiate(&gexec, g, 0);
        cudaGraphDestroy(g);
        graph_steps = steps_per_graph;
        return e;
    }
};

namespace {
thread_local std::string g_batch_err;
int berr(plbm_batch *b, int code, const std::string &m)
{
    if (b) b->err = m;
    g_batch_err = m;
    return code;
}
}  // namespace

extern "C" {

int plbm_batch_create(unsigned n, const plbm_batch_domain *doms, int precision, plbm_batch **out)
{
    if (!doms || !out || n == 0) return berr(nullptr, PLBM_ERR_ARGUMENT, "plbm_batch_create: no domains");
    if (precision != PLBM_F32 && precision != PLBM_F16S && precision != PLBM_BF16S && precision != PLBM_F64_Q60 &&
        precision != PLBM_F16C)
        return berr(nullptr, PLBM_ERR_ARGUMENT,
                    "batches support PLBM_F32, PLBM_F16S, PLBM_BF16S, PLBM_F16C and PLBM_F64_Q60");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return berr(nullptr, PLBM_ERR_NO_DEVICE, "no CUDA device");
    auto *b = new plbm_batch();
    b->prec = precision;
    if (cudaMalloc(&b->status_pending, sizeof(int)) != cudaSuccess) {
        delete b;
        return berr(nullptr, PLBM_ERR_CUDA, "cudaMalloc status");
    }
    b->status_d = b->status_pending;
    auto fail = [&](cudaError_t e, const char *what) {
        const int rc = berr(b, PLBM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
        delete b;
        return rc;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail(e, "stream");
    const bool shifted = precision != PLBM_F64_Q60;
    const size_t eb = precision == PLBM_F32 ? 4 : precision == PLBM_F64_Q60 ? 8 : 2;
    std::vector<int8_t> flags_host;
    for (unsigned i = 0; i < n; ++i) {
        const plbm_batch_domain &s = doms[i];
        if (s.inner_w < 2 || s.inner_h < 3 || !(s.relaxation_time > 0.5) || !s.mask) {
            delete b;
            return berr(nullptr, PLBM_ERR_ARGUMENT, "domain " + std::to_string(i) + ": need W >= 2, H >= 3, tau > 0.5, a mask");
        }
        StepParams d;
        std::memset(&d, 0, sizeof d);
        d.W = (int)s.inner_w; d.H = (int)s.inner_h; d.P = (d.W + 31) / 32 * 32;
        d.N = (unsigned long long)d.P * d.H;
        b->nodes += (unsigned long long)d.W * d.H;
        plbm::maxwell_boltzmann<double>(0, 0, 1, d.weight);
        plbm::maxwell_boltzmann<double>(0, 0, s.inlet_density, d.feq_in);
        plbm::maxwell_boltzmann<double>(0, 0, s.outlet_density, d.feq_out);
        d.omega = 1 / s.relaxation_time;
        d.rho_out = s.outlet_density;
        plbm::fill_float_constants(d, shifted, true, s.inlet_density, s.outlet_density,
                                   precision == PLBM_F16S ? (double)plbm::F16_SCALE : 1.0);
        plbm::fill_q60_constants(d);
        // device buffers of the domain
        int8_t *flags = nullptr;
        void *ptrs[8] = {};
        size_t sizes[8] = { 9 * d.N * eb, 9 * d.N * eb, d.N * 2, (size_t)d.W * d.H, 4 * (size_t)d.W * d.H * 8,
                            2 * (size_t)d.H * 8, 0, 0 };
        for (int k = 0; k < 6; ++k) {
            e = cudaMalloc(&ptrs[k], sizes[k]);
            if (e != cudaSuccess) return fail(e, "cudaMalloc domain");
            b->allocs.push_back(ptrs[k]);
        }
        d.links = (const uint16_t *)ptrs[2];
        flags = (int8_t *)ptrs[3];
        double *res = (double *)ptrs[4];
        d.rho = res; d.jx = res + (size_t)d.W * d.H; d.jy = res + 2 * (size_t)d.W * d.H; d.jabs = res + 3 * (size_t)d.W * d.H;
        double *jyc = (double *)ptrs[5];
        d.nan_protection = 1;
        d.status = b->status_pending;
        d.lat_elems = 9ull * d.N;
        e = cudaMemcpyAsync(flags, s.mask, (size_t)d.W * d.H, cudaMemcpyHostToDevice, b->stream);
        if (e == cudaSuccess) e = plbm::launch_links(flags, (uint16_t *)ptrs[2], d.W, d.H, d.P, b->stream);
        double rest[9];
        for (int k = 0; k < 9; ++k) rest[k] = d.weight[k];
        for (int k = 0; k < 2 && e == cudaSuccess; ++k)
            e = shifted ? plbm::launch_fill_shifted(ptrs[k], precision, plbm::STREAM, d.P, d.N, rest, d.shift_a, d.shift_g,
                                                    b->stream)
                        : plbm::launch_fill_lattice(ptrs[k], precision, plbm::STREAM, d.N, rest, b->stream);
        if (e == cudaSuccess) e = plbm::launch_fill_results(d.rho, d.jx, d.jy, d.jabs, (unsigned long long)d.W * d.H, b->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(jyc, 0, 2 * (size_t)d.H * 8, b->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);   // the mask buffer is the caller's
        if (e != cudaSuccess) return fail(e, "domain set-up");
        for (unsigned par = 0; par < 2; ++par) {
            StepParams q = d;
            q.lat0 = ptrs[par];
            q.lat1 = ptrs[par ^ 1u];
            q.jy_prev = jyc + (size_t)par * d.H;
            q.jy_next = jyc + (size_t)(par ^ 1u) * d.H;
            b->host.push_back(q);
        }
    }
    e = cudaMalloc(&b->dom_d, b->host.size() * sizeof(StepParams));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->dom_d, b->host.data(), b->host.size() * sizeof(StepParams), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaMalloc(&b->ticket_d, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemsetAsync(b->status_d, 0, sizeof(int), b->stream);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    b->blocks = sms * 8;
    if (e == cudaSuccess) e = b->build_tiles();
    if (e != cudaSuccess) return fail(e, "batch set-up");
    *out = b;
    return PLBM_OK;
}

void plbm_batch_destroy(plbm_batch *b) { delete b; }

int plbm_batch_set_tile(plbm_batch *b, int tile_w, int tile_h, int blocks_per_sm)
{
    // tile_h carries the rows each thread sweeps and the vectorised-rows flag in its upper bits:
    // tile_h = threads_y + 256 * rows (+ PLBM_BATCH_TILE_VEC)
    const int ty = tile_h & 255, rows = std::max(1, (tile_h >> 8) & 255);
    const bool v = (tile_h & PLBM_BATCH_TILE_VEC) != 0;
    // k_batch / k_batch_vec are compiled for at most 256 threads per block (__launch_bounds__)
    if (tile_w < 1 || ty < 1 || tile_w * ty > 256 || blocks_per_sm < 1)
        return berr(b, PLBM_ERR_ARGUMENT, "tile must have 1..256 threads and blocks_per_sm >= 1");
    if (v && (!b->two_byte() || tile_w != 32 || ty > 8))
        return berr(b, PLBM_ERR_ARGUMENT,
                    "vectorised rows: PLBM_F16S / PLBM_BF16S / PLBM_F16C batches, tiles of 32 x (1..8) threads");
    b->vec_rows = v;
    b->tile_w = tile_w;
    b->tile_h = ty;
    b->tile_rows = rows;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    b->blocks = sms * blocks_per_sm;
    const cudaError_t e = b->build_tiles();
    return e == cudaSuccess ? PLBM_OK : berr(b, PLBM_ERR_CUDA, cudaGetErrorString(e));
}

int plbm_batch_run(plbm_batch *b, unsigned steps, int mode, double *ms_per_step)
{
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaError_t e = cudaEventRecord(e0, b->stream);
    const unsigned per_graph = 16;
    unsigned k = 0;
    if (mode == PLBM_BATCH_PERSISTENT_GRAPH && steps >= per_graph) {
        if ((b->t & 1u) && e == cudaSuccess) { e = b->launch(b->t, 0); ++k; }
        if (e == cudaSuccess) e = b->ensure_graph(per_graph);
        while (e == cudaSuccess && k + per_graph <= steps - 1) {
            e = cudaGraphLaunch(b->gexec, b->stream);
            k += per_graph;
        }
    }
    for (; k < steps && e == cudaSuccess; ++k) {
        const int last = k + 1 == steps;
        e = mode == PLBM_BATCH_PER_DOMAIN ? b->launch_per_domain(b->t + k, last) : b->launch(b->t + k, last);
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return berr(b, PLBM_ERR_CUDA, cudaGetErrorString(e));
    b->t += steps;
    if (ms_per_step) *ms_per_step = steps ? ms / steps : 0.0;
    int st = 0;
    cudaMemcpy(&st, b->status_d, sizeof(int), cudaMemcpyDeviceToHost);
    if (st & plbm::STATUS_OUT_OF_RANGE)
        return berr(b, PLBM_ERR_CUDA, "checked build: a batch kernel computed an index outside its buffer");
    if (st)
        return berr(b, PLBM_ERR_NUMERIC, b->prec == PLBM_F16C ? "a population deviation left the f16c range"
                                                              : "a population left the f64_q60 range");
    return PLBM_OK;
}

int plbm_batch_autotune(plbm_batch *b, unsigned steps, int *tile_w, int *tile_h, int *blocks_per_sm)
{
    // threads_x, threads_y + 256 * rows swept per thread
    static const int cand[][2] = { { 32, 4 + 256 * 1 }, { 32, 4 + 256 * 4 }, { 32, 4 + 256 * 8 }, { 32, 8 + 256 * 4 },
                                   { 64, 2 + 256 * 8 }, { 64, 4 + 256 * 4 }, { 128, 2 + 256 * 4 } };
    // 2-byte batches also try vectorised rows (fast in open channels; porous domains send many
    // nodes through the scalar edge gather and favour one node per thread)
    static const int cand_vec[][2] = { { 32, 4 + 256 * 1 }, { 32, 4 + 256 * 2 }, { 32, 4 + 256 * 4 }, { 32, 8 + 256 * 1 },
                                       { 32, 8 + 256 * 2 }, { 32, 2 + 256 * 4 }, { 32, 2 + 256 * 8 } };
    static const int bps[] = { 4, 8, 16 };
    static const int bps_vec[] = { 2, 4, 8 };
    double best = 1e300;
    int bw = b->tile_w, bh = b->tile_h + 256 * b->tile_rows + (b->vec_rows ? PLBM_BATCH_TILE_VEC : 0), bb = 8;
    auto tryit = [&](int w, int h, int k) {
        if (plbm_batch_set_tile(b, w, h, k) != PLBM_OK) return PLBM_OK;
        double ms = 0;
        if (plbm_batch_run(b, steps, PLBM_BATCH_PERSISTENT, &ms) != PLBM_OK) return PLBM_ERR_CUDA;
        if (ms < best) { best = ms; bw = w; bh = h; bb = k; }
        return PLBM_OK;
    };
    for (const auto &c : cand)
        for (int k : bps)
            if (tryit(c[0], c[1], k) != PLBM_OK) return PLBM_ERR_CUDA;
    if (b->two_byte())
        for (const auto &c : cand_vec)
            for (int k : bps_vec)
                if (tryit(c[0], c[1] + PLBM_BATCH_TILE_VEC, k) != PLBM_OK) return PLBM_ERR_CUDA;
    const int rc = plbm_batch_set_tile(b, bw, bh, bb);
    if (tile_w) *tile_w = bw;
    if (tile_h) *tile_h = bh;   // threads_y + 256 * rows
    if (blocks_per_sm) *blocks_per_sm = bb;
    return rc;
}

int plbm_batch_results(plbm_batch *b, unsigned domain, int which, double *out)
{
    if (domain >= b->n_domains() || which < 0 || which > 3) return berr(b, PLBM_ERR_ARGUMENT, "bad domain/which");
    const StepParams &d = b->host[2 * domain];
    const double *src = which == 0 ? d.rho : which == 1 ? d.jx : which == 2 ? d.jy : d.jabs;
    // on the batch's own (non-blocking) stream, so the copy is ordered after its steps
    cudaError_t e = cudaMemcpyAsync(out, src, (size_t)d.W * d.H * 8, cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    return e == cudaSuccess ? PLBM_OK : berr(b, PLBM_ERR_CUDA, cudaGetErrorString(e));
}

int plbm_batch_info(plbm_batch *b, unsigned long long *nodes, unsigned *tiles)
{
    if (nodes) *nodes = b->nodes;
    if (tiles) *tiles = b->n_tiles;
    return PLBM_OK;
}

const char *plbm_batch_last_error(void) { return g_batch_err.c_str(); }

}  // extern "C"
