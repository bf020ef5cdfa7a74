/*
 * plbm_oracle.c — CPU restatement of PortLBM's per-timestep D2Q9 BGK update.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  Nothing in the product library links or
 * calls this file; tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * use it as the checker.
 *
 * The restatement is literal: each step runs the reference's kernels one after the
 * other (bounce-back emplacement, outlet update, stream/collide, lattice swap), with
 * the reference's node/layout index arithmetic in 32-bit unsigned integers, its
 * per-algorithm padded or buffered domains, and its one-lattice buffer refreshes.
 * Reference citations are paths inside the SC-SGS/PortLBM project.
 *
 * Build with -ffp-contract=off: the floating-point expressions below are written in
 * the same order and with the same C/C++ promotion rules as the reference, so the
 * executed IEEE operations are the reference's.  -DPLBMO_FLOAT restates the
 * reference's USE_FLOAT build (include/lbm/core/constants.hpp:17-21).
 */
#include "plbm_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef PLBMO_FLOAT
typedef float real;
#else
typedef double real;
#endif

/* include/lbm/core/constants.hpp:38-39 — double expressions converted to real_type. */
static const real W[9] = { 1.0 / 36, 1.0 / 9,  1.0 / 36, 1.0 / 9, 4.0 / 9,
                           1.0 / 9,  1.0 / 36, 1.0 / 9,  1.0 / 36 };

struct plbmo_sim {
    int alg, layout, nan_protection;
    unsigned X, V;          /* Properties::horizontal_nodes / vertical_nodes (inner + 2) */
    plbmo_domain dom;
    unsigned N;             /* nodes per lattice (Data's total_node_count) */
    unsigned Hs;            /* horizontal stride of the stored grid */
    int8_t *flags;          /* Data::phase_information: -1 ghost/pad/buffer, 0 fluid, 1 solid */
    real *lat[2];           /* distribution_values_0 / _1 (two-lattice only for [1]) */
    real *res[4];           /* Results: densities, x/y "velocities" (momentum), |j| */
    unsigned nres;
    real omega;             /* relaxation_time_inverse = 1 / relaxation_time */
    real rho_out;
};

/* ---- include/lbm/core/access.hpp ------------------------------------------------------ */

/* CollisionAccessor::at :117-121, StreamAccessor::at :142-146, BundleAccessor::at :167-171 */
static inline unsigned at(int layout, unsigned node, unsigned d, unsigned n_total)
{
    if (layout == PLBMO_COLLISION) return 9u * node + d;
    if (layout == PLBMO_STREAM) return n_total * d + node;
    return 3u * (d / 3u) * n_total + (d % 3u) + 3u * node;
}

/* get_neighbor :203-213 (unsigned wrap-around arithmetic as in the reference) */
static inline unsigned nb(unsigned node, unsigned d, unsigned h)
{
    int y_off = (int)(d / 3) - 1;
    int x_off = (int)(d % 3) - 1;
    return node + (unsigned)(y_off * (int)h) + (unsigned)x_off;
}

/* get_result_index(x, y, horizontal_nodes_domain) :269-273 */
static inline unsigned result_index(unsigned x, unsigned y, unsigned X) { return (x - 1) + (y - 1) * (X - 2); }

/* NonBufferedNodeAccess::get_index :321-329 and BufferedNodeAccess::get_index :353-362 */
static inline unsigned node_index(const plbmo_sim *s, unsigned x, unsigned y)
{
    if (s->alg == PLBMO_NPOL || s->alg == PLBMO_NSOL)
        return (x + ((x - 1) / s->dom.subdomain_horizontal_nodes))
               + (y + ((y - 1) / s->dom.subdomain_vertical_nodes)) * s->dom.horizontal_nodes;
    return x + y * s->dom.horizontal_nodes;
}

/* ---- include/lbm/core/simulation.hpp:373-446, src/lbm/core/simulation.cpp:223-382 ----- */

static size_t which_power_of_4(size_t x)
{
    size_t checkbit = 3, pow = 0;
    if (x & 0x1) return 0;
    if (x == 0) return 0; /* the reference loops forever here; validate() rejects 0 first */
    while (!(checkbit & x)) { x >>= 2; pow++; }
    return !(x & 2) ? pow : 0;
}

static size_t which_power_of_2(size_t x)
{
    size_t checkbit = 1, pow = 0;
    if (x & 0x1) return 0;
    if (x == 0) return 0;
    while (!(checkbit & x)) { x >>= 1; pow++; }
    return !(x >> 1 | 0) ? pow : 0;
}

/* power_of_two_handling simulation.cpp:223-261 */
static void power_of_two_handling(size_t wg, unsigned *sv, unsigned *sh)
{
    size_t p4 = which_power_of_4(wg), p2 = which_power_of_2(wg);
    if (p4) {
        size_t size = 1;
        for (size_t i = 0; i < p4; ++i) size *= 2;
        *sh = (unsigned)size; *sv = (unsigned)size;
    } else if (p2) {
        size_t ph = p2 / 2, height = 1;
        for (size_t i = 0; i < ph; ++i) height *= 2;
        *sv = (unsigned)height; *sh = (unsigned)(2 * height);
    } else {
        *sv = 2; *sh = (unsigned)(wg / 2);
    }
}

static void counts(unsigned ext, unsigned sub, unsigned *count)
{
    *count = ((ext - 2) / sub) + 1;
    if (!((ext - 2) % sub)) (*count)--;
}

int plbmo_domain_for(int algorithm, unsigned wg, unsigned X, unsigned V, plbmo_domain *d)
{
    /* Domain(Properties&) :194-221 defaults, then per-algorithm setup */
    d->total_node_count = X * V; d->vertical_nodes = V; d->horizontal_nodes = X;
    d->subdomain_vertical_nodes = V; d->subdomain_horizontal_nodes = X;
    d->subdomain_count_vertical = 1; d->subdomain_count_horizontal = 1;
    if (algorithm == PLBMO_LPTL) return 0;
    unsigned sv, sh;
    size_t w = wg;
    if (algorithm == PLBMO_NSOL) {           /* setup_for_swap :329-382 */
        if (w < 6) return -1;
        if (w & 0x1) w--;
        power_of_two_handling(w, &sv, &sh);
        sv -= 1; sh -= 2;
        /* the power-of-4 branch can give 2x2 tiles (wg 20, 36, ...): the reference then divides by
           zero in the subdomain count; report it instead */
        if (sh == 0 || sv == 0) return -1;
    } else if (w & 0x1) {                    /* :268-273 / :301-306 */
        sh = (unsigned)w; sv = 1;
    } else {
        power_of_two_handling(w, &sv, &sh);
    }
    d->subdomain_vertical_nodes = sv; d->subdomain_horizontal_nodes = sh;
    counts(V, sv, &d->subdomain_count_vertical);
    counts(X, sh, &d->subdomain_count_horizontal);
    if (algorithm == PLBMO_NPTL) {           /* setup_for_decomposed_two_lattice :263-294 */
        d->vertical_nodes = sv * d->subdomain_count_vertical + 2;
        d->horizontal_nodes = sh * d->subdomain_count_horizontal + 2;
    } else {                                 /* setup_for_buffered_two_lattice :296-327, swap :367-381 */
        d->vertical_nodes = (sv + 1) * d->subdomain_count_vertical + 1;
        d->horizontal_nodes = (sh + 1) * d->subdomain_count_horizontal + 1;
    }
    d->total_node_count = d->vertical_nodes * d->horizontal_nodes;
    return 0;
}

/* ---- glibc random() TYPE_3 (the sequence behind an unseeded std::rand()) -------------------
 * Published algorithm: r[0] = seed; r[i] = 16807 * r[i-1] mod (2^31 - 1) for i = 1..30;
 * r[i] = r[i-31] for i = 31..33; r[i] = r[i-31] + r[i-3] (mod 2^32) for i >= 34; the k-th
 * output is r[k + 344] >> 1.  domain_initialization.hpp:277-278 draws from it. */
static uint32_t g_ring[34];
static unsigned g_pos;

void plbmo_rand_reset(unsigned seed)
{
    int32_t r0 = (int32_t)(seed == 0 ? 1 : seed);
    g_ring[0] = (uint32_t)r0;
    for (int i = 1; i < 31; ++i) {
        long long v = (16807LL * (long long)(int32_t)g_ring[i - 1]) % 2147483647LL;
        if (v < 0) v += 2147483647LL;
        g_ring[i] = (uint32_t)v;
    }
    for (int i = 31; i < 34; ++i) g_ring[i] = g_ring[i - 31];
    g_pos = 34;
    for (int i = 34; i < 344; ++i) (void)plbmo_rand();
}

int plbmo_rand(void)
{
    uint32_t v = g_ring[(g_pos - 31) % 34] + g_ring[(g_pos - 3) % 34];
    g_ring[g_pos % 34] = v;
    g_pos++;
    return (int)(v >> 1);
}

/* ---- include/lbm/core/domain_initialization.hpp ------------------------------------------ */

/* Stencils :41-192; arguments are stored extents X (horizontal) and V (vertical). */
static unsigned stencil(int scenario, unsigned x, unsigned y, unsigned V, unsigned X)
{
    switch (scenario) {
    case PLBMO_HAGEN_POISEUILLE: return 0;
    case PLBMO_WALLS: { /* :59-72 */
        unsigned cond = (x == (1 * X) / 6 || x == (3 * X) / 6 || x == (5 * X) / 6) && (y > 1) && (y < V / 2);
        cond += (x == (2 * X) / 6 || x == (4 * X) / 6) && (y < V - 2) && (y > ((V - 1) / 2));
        return cond;
    }
    case PLBMO_CIRCLE: { /* :80-94 — unsigned differences; abs of an unsigned is the identity */
        unsigned mx = 2 * X / 10, my = V / 2, r = V / 5;
        unsigned dx = mx - x, dy = my - y;
        return (y >= my - r) && (y <= my + r) && (x >= mx - r) && (x <= mx + r) && (dx * dx + dy * dy <= r * r);
    }
    case PLBMO_SQUARE: { /* :102-114 */
        unsigned mx = 2 * X / 10, my = V / 2, hl = V / 10;
        return (y >= my - hl) && (y <= my + hl) && (x >= mx - hl) && (x <= mx + hl);
    }
    case PLBMO_PLATE: { /* :122-135 */
        unsigned mx = X / 10, my = V / 2, hh = 7 * V / 40, hw = hh / 60;
        return (y >= my - hh) && (y <= my + hh) && (x >= mx - hw) && (x <= mx + hw);
    }
    case PLBMO_SKYSCRAPER: { /* :144-165, with C's && / || precedence exactly as written */
        unsigned ha = V / 2, hwa = 1, hs = 2 * V / 5, hws = V / 24, hf = V / 4, hwf = V / 16, mx = 3 * X / 10;
        return ((y >= 1) && (y <= hf && x >= mx - hwf && x <= mx + hwf))
               || (y <= hs && x >= mx - hws && x <= mx + hws)
               || (y <= ha && x >= mx - hwa && x <= mx + hwa);
    }
    case PLBMO_WING: { /* :173-191 — int centre converted to unsigned in x - middle_x */
        int mx = (int)(X / 5), my = (int)(V / 2), rmax = (int)(V / 5), sy = 5;
        unsigned ddx = x - (unsigned)mx, ddy = y - (unsigned)my;
        unsigned c = ((0.2 * (double)(ddx * ddx) + (double)(ddy * ddy)) <= rmax)
                     || ((pow((double)ddx, 1.4) + (double)((unsigned)(sy * sy) * (ddy * ddy))) <= sy * sy * rmax);
        return c;
    }
    default: return 0;
    }
}

/* maxwell_boltzmann_distribution simulation.hpp:333-350 (std::pow(v, 2) promotes to double) */
static void maxwell_boltzmann(real ux, real uy, real rho, real *t)
{
    for (int d = 0; d < 9; ++d) {
        int vx = (d % 3) - 1, vy = (d / 3) - 1;
        t[d] = W[d] * (rho + 3 * (vx * ux + vy * uy) + 9.0 / 2 * pow((double)(vx * ux + vy * uy), 2)
                       - 3.0 / 2 * (ux * ux + uy * uy));
    }
}

/* ---- step kernels ----------------------------------------------------------------------- */

#define S_AT(n, d) at(s->layout, (n), (d), s->N)

/* EmplaceBounceBackKernel nptl_kernels.hpp:471-491 (lptl :451-467, npol :232-253, nsol :81-102):
 * solid node s, d != 4: S[s][d] = S[s + c_d][8 - d] in the source lattice. */
static void emplace_one(plbmo_sim *s, real *S, unsigned n)
{
    if (s->flags[n] == 1) {
        for (unsigned d = 0; d < 4; ++d) S[S_AT(n, d)] = S[S_AT(nb(n, d, s->Hs), 8 - d)];
        for (unsigned d = 5; d < 9; ++d) S[S_AT(n, d)] = S[S_AT(nb(n, d, s->Hs), 8 - d)];
    }
}

static void emplace(plbmo_sim *s, real *S)
{
    const plbmo_domain *D = &s->dom;
    if (s->alg == PLBMO_LPTL) {              /* range<1>(V*X) lptl.hpp:86-88 */
        long n_all = (long)s->N;
#pragma omp parallel for schedule(static)
        for (long n = 0; n < n_all; ++n) emplace_one(s, S, (unsigned)n);
    } else if (s->alg == PLBMO_NPTL) {       /* nd_range({Vexp-2, Hexp-2}) nptl.hpp:88-91 */
        long rows = (long)D->vertical_nodes - 2;
#pragma omp parallel for schedule(static)
        for (long gy = 0; gy < rows; ++gy)
            for (unsigned gx = 0; gx < D->horizontal_nodes - 2; ++gx)
                emplace_one(s, S, (gx + 1) + ((unsigned)gy + 1) * D->horizontal_nodes);
    } else {                                 /* nd_range({sv*cv, sh*ch}) over BufferedNodeAccess npol.hpp:139-146 */
        long rows = (long)D->subdomain_vertical_nodes * D->subdomain_count_vertical;
        unsigned cols = D->subdomain_horizontal_nodes * D->subdomain_count_horizontal;
#pragma omp parallel for schedule(static)
        for (long gy = 0; gy < rows; ++gy)
            for (unsigned gx = 0; gx < cols; ++gx)
                emplace_one(s, S, node_index(s, gx + 1, (unsigned)gy + 1));
    }
}

/* HorizontalCopyToBufferKernel buffered.hpp:74-93 and VerticalCopyToBufferKernel :133-152 */
static void refresh_buffers(plbmo_sim *s, real *S)
{
    const plbmo_domain *D = &s->dom;
    unsigned H = D->horizontal_nodes;
    if (D->subdomain_count_vertical > 1) {
        for (unsigned i = 0; i + 1 < D->subdomain_count_vertical; ++i)
            for (unsigned x = 0; x < H; ++x) {
                unsigned y = (i + 1) * (D->subdomain_vertical_nodes + 1);
                unsigned n = x + y * H, top = nb(n, 7, H), bottom = nb(n, 1, H);
                for (unsigned d = 0; d < 3; ++d) S[S_AT(n, d)] = S[S_AT(top, d)];
                for (unsigned d = 6; d < 9; ++d) S[S_AT(n, d)] = S[S_AT(bottom, d)];
            }
    }
    if (D->subdomain_count_horizontal > 1) {
        for (unsigned y = 0; y < D->vertical_nodes; ++y)
            for (unsigned j = 0; j + 1 < D->subdomain_count_horizontal; ++j) {
                unsigned x = (j + 1) * (D->subdomain_horizontal_nodes + 1);
                unsigned n = x + y * H, left = nb(n, 3, H), right = nb(n, 5, H);
                for (unsigned d = 2; d < 9; d += 3) S[S_AT(n, d)] = S[S_AT(left, d)];
                for (unsigned d = 0; d < 9; d += 3) S[S_AT(n, d)] = S[S_AT(right, d)];
            }
    }
}

/* OutletUpdateKernel non_buffered.hpp:75-130 and buffered.hpp:268-326 (border located as
 * BufferedNodeAccess(X-3, y) + 1 in the buffered variant, literally). */
static void outlet(plbmo_sim *s, real *S)
{
    unsigned H = s->Hs, X = s->X;
    for (unsigned id = 0; id + 4 < s->V; ++id) {
        unsigned y = id + 2;
        unsigned b;
        if (s->alg == PLBMO_NPOL || s->alg == PLBMO_NSOL) b = nb(node_index(s, X - 3, y), 5, H);
        else b = (X - 2) + y * H;
        real f1 = S[S_AT(nb(b, 7, H), 1)];
        real f4 = S[S_AT(b, 4)];
        real f7 = S[S_AT(nb(b, 1, H), 7)];
        real fi[3];
        for (unsigned i = 0; i < 3; ++i) fi[i] = S[S_AT(nb(b, 3 * i, H), 8 - 3 * i)];
        real xv = -s->rho_out + (f1 + f4 + f7 + 2 * (fi[0] + fi[1] + fi[2]));
        real yv = s->res[2][result_index(X - 3, y, X)];
        S[S_AT(nb(b, 8, H), 0)] = fi[0] - 0.5 * (f1 - f7) - 1.0 / 6 * xv - 0.5 * yv;
        S[S_AT(nb(b, 5, H), 3)] = fi[1] - (2.0 / 3) * xv;
        S[S_AT(nb(b, 2, H), 6)] = fi[2] + 0.5 * (f1 - f7) - 1.0 / 6 * xv + 0.5 * yv;
    }
}

/* Moments + BGK of StreamCollideKernel nptl_kernels.hpp:381-437 (identical in lptl :357-412,
 * npol :136-197, nsol :277-332).  Writes the 9 post-collision values to out[] and the
 * macroscopic observables to the results at index r. */
static inline void collide_node(plbmo_sim *s, const real f[9], real out[9], unsigned r)
{
    real density = 0, fvx = 0, fvy = 0, absv = 0, rb = 0, result = 0;
    int vx = 0, vy = 0;
    for (int d = 0; d < 9; ++d) {
        density += f[d];
        vx = d % 3 - 1; vy = d / 3 - 1;
        fvx += f[d] * vx;
        fvy += f[d] * vy;
    }
    absv = fvx * fvx + fvy * fvy;
    for (int d = 0; d < 9; ++d) {
        vx = (d % 3) - 1; vy = (d / 3) - 1;
        rb = vx * fvx + vy * fvy;
        result = W[d] * (density + 3 * rb + 9.0 / 2 * rb * rb - 3.0 / 2 * absv);
        result = -s->omega * (f[d] - result) + f[d];
        out[d] = result;
    }
    absv = sqrt(absv);
    if (s->nan_protection) { /* WITH_NAN_PROTECTION :413-432 */
        if (isnan(density) || density > FLT_MAX) density = 0;
        if (isnan(fvx) || fvx > FLT_MAX) fvx = 0;
        if (isnan(fvy) || fvy > FLT_MAX) fvy = 0;
        if (isnan(absv) || absv > FLT_MAX) absv = 0;
    }
    s->res[0][r] = density; s->res[1][r] = fvx; s->res[2][r] = fvy; s->res[3][r] = absv;
}

/* nptl StreamCollideKernel :350-439 over nd_range({Vexp-2, Hexp-2}); lptl :331-414 over range(V*X). */
static void stream_collide_two_lattice(plbmo_sim *s, const real *S, real *Dst)
{
    unsigned H = s->Hs;
    if (s->alg == PLBMO_LPTL) {
        long n_all = (long)s->N;
#pragma omp parallel for schedule(static)
        for (long ln = 0; ln < n_all; ++ln) {
            unsigned n = (unsigned)ln;
            if (!s->flags[n]) {
                /* get_result_index(node, horizontal_nodes) access.hpp:286-290 */
                unsigned r = (((n - H) / H) * (H - 2) + (n - 1) % H);
                real f[9], o[9];
                for (unsigned d = 0; d < 9; ++d) f[d] = S[S_AT(nb(n, 8 - d, H), d)];
                collide_node(s, f, o, r);
                for (unsigned d = 0; d < 9; ++d) Dst[S_AT(n, d)] = o[d];
            }
        }
        return;
    }
    long rows = (long)s->dom.vertical_nodes - 2;
#pragma omp parallel for schedule(static)
    for (long gy = 0; gy < rows; ++gy)
        for (unsigned gx = 0; gx < s->dom.horizontal_nodes - 2; ++gx) {
            unsigned x = gx + 1, y = (unsigned)gy + 1, n = x + y * H;
            if (!s->flags[n]) {
                unsigned r = result_index(x, y, s->X);
                real f[9], o[9];
                for (unsigned d = 0; d < 9; ++d) f[d] = S[S_AT(nb(n, 8 - d, H), d)];
                collide_node(s, f, o, r);
                for (unsigned d = 0; d < 9; ++d) Dst[S_AT(n, d)] = o[d];
            }
        }
}

/* npol StreamCollideKernel npol_kernels.hpp:89-199: per work-group, every item pulls its 9
 * values, barrier, then fluid items write in place.  Work-groups run one at a time here; the
 * buffer lines make them independent. */
static void stream_collide_npol(plbmo_sim *s, real *S)
{
    const plbmo_domain *D = &s->dom;
    unsigned H = s->Hs, sv = D->subdomain_vertical_nodes, sh = D->subdomain_horizontal_nodes;
    long groups = (long)D->subdomain_count_vertical * D->subdomain_count_horizontal;
#pragma omp parallel
    {
        real *p = (real *)malloc(sizeof(real) * 9 * (size_t)sv * sh);
#pragma omp for schedule(static)
        for (long g = 0; g < groups; ++g) {
            unsigned ty = (unsigned)(g / D->subdomain_count_horizontal), tx = (unsigned)(g % D->subdomain_count_horizontal);
            for (unsigned ly = 0; ly < sv; ++ly)
                for (unsigned lx = 0; lx < sh; ++lx) {
                    unsigned g1 = tx * sh + lx, g0 = ty * sv + ly;
                    unsigned x = g1 + 1 + g1 / sh, y = g0 + 1 + g0 / sv, n = x + y * H;
                    if (!s->flags[n])
                        for (unsigned d = 0; d < 9; ++d) p[9 * (ly * sh + lx) + d] = S[S_AT(nb(n, 8 - d, H), d)];
                }
            for (unsigned ly = 0; ly < sv; ++ly)
                for (unsigned lx = 0; lx < sh; ++lx) {
                    unsigned g1 = tx * sh + lx, g0 = ty * sv + ly;
                    unsigned x = g1 + 1 + g1 / sh, y = g0 + 1 + g0 / sv, n = x + y * H;
                    if (!s->flags[n]) {
                        unsigned r = result_index(x - x / (sh + 1), y - y / (sv + 1), s->X);
                        real o[9];
                        collide_node(s, &p[9 * (ly * sh + lx)], o, r);
                        for (unsigned d = 0; d < 9; ++d) S[S_AT(n, d)] = o[d];
                    }
                }
        }
        free(p);
    }
}

/* nsol StreamCollideKernel nsol_kernels.hpp:171-334 with its local-memory exchange restated:
 * items send their own 5,6 then 7,8 values to neighbour slots, pull 3,2 then 1,0 from
 * global memory, and collect 5,6 then 7,8 from their own slot after barriers. */
static void stream_collide_nsol(plbmo_sim *s, real *S)
{
    const plbmo_domain *D = &s->dom;
    unsigned H = s->Hs, sv = D->subdomain_vertical_nodes, sh = D->subdomain_horizontal_nodes;
    unsigned lrx = sh + 2, lry = sv + 1, bw = sh + 4;
    size_t local_len = 2 * (size_t)(sh + 4) * (sv + 2);
    long groups = (long)D->subdomain_count_vertical * D->subdomain_count_horizontal;
#pragma omp parallel
    {
        real *local = (real *)calloc(local_len, sizeof(real));
        real *p = (real *)calloc(9 * (size_t)lrx * lry, sizeof(real));
#pragma omp for schedule(static)
        for (long g = 0; g < groups; ++g) {
            unsigned ty = (unsigned)(g / D->subdomain_count_horizontal), tx = (unsigned)(g % D->subdomain_count_horizontal);
            memset(local, 0, local_len * sizeof(real));
#define ITEM_SETUP                                                                   \
    unsigned g1 = tx * lrx + lx, g0 = ty * lry + ly;                                 \
    unsigned x = g1 - g1 / lrx, y = g0, n = x + y * H;                               \
    unsigned own = (lx + 1) + ly * bw;                                               \
    real *pp = &p[9 * (ly * lrx + lx)];                                              \
    (void)own; (void)pp; (void)n
            for (unsigned ly = 0; ly < lry; ++ly)
                for (unsigned lx = 0; lx < lrx; ++lx) {
                    ITEM_SETUP;
                    pp[4] = S[S_AT(n, 4)];
                    local[2 * nb(own, 5, bw)] = S[S_AT(n, 5)];
                    pp[3] = S[S_AT(nb(n, 5, H), 3)];
                    local[2 * nb(own, 6, bw) + 1] = S[S_AT(n, 6)];
                    pp[2] = S[S_AT(nb(n, 6, H), 2)];
                }
            for (unsigned ly = 0; ly < lry; ++ly)
                for (unsigned lx = 0; lx < lrx; ++lx) {
                    ITEM_SETUP;
                    pp[5] = local[2 * own];
                    pp[6] = local[2 * own + 1];
                }
            for (unsigned ly = 0; ly < lry; ++ly)
                for (unsigned lx = 0; lx < lrx; ++lx) {
                    ITEM_SETUP;
                    local[2 * nb(own, 7, bw)] = S[S_AT(n, 7)];
                    pp[1] = S[S_AT(nb(n, 7, H), 1)];
                    local[2 * nb(own, 8, bw) + 1] = S[S_AT(n, 8)];
                    pp[0] = S[S_AT(nb(n, 8, H), 0)];
                }
            for (unsigned ly = 0; ly < lry; ++ly)
                for (unsigned lx = 0; lx < lrx; ++lx) {
                    ITEM_SETUP;
                    pp[7] = local[2 * own];
                    pp[8] = local[2 * own + 1];
                    if (!s->flags[n]) {
                        unsigned r = result_index(x - x / (sh + 1), y - y / (sv + 1), s->X);
                        real o[9];
                        collide_node(s, pp, o, r);
                        for (unsigned d = 0; d < 9; ++d) S[S_AT(n, d)] = o[d];
                    }
                }
#undef ITEM_SETUP
        }
        free(local);
        free(p);
    }
}

/* Per-step drivers: nptl.hpp:121-134, lptl.hpp:117-130, npol.hpp:185-194 (emplace_bounce_back
 * :122-159), nsol.hpp:189-198. */
void plbmo_run(plbmo_sim *s, unsigned steps)
{
    for (unsigned t = 0; t < steps; ++t) {
        if (s->alg == PLBMO_NPTL || s->alg == PLBMO_LPTL) {
            emplace(s, s->lat[0]);
            outlet(s, s->lat[0]);
            stream_collide_two_lattice(s, s->lat[0], s->lat[1]);
            real *tmp = s->lat[1]; s->lat[1] = s->lat[0]; s->lat[0] = tmp;
        } else {
            refresh_buffers(s, s->lat[0]);
            emplace(s, s->lat[0]);
            refresh_buffers(s, s->lat[0]);
            outlet(s, s->lat[0]);
            if (s->alg == PLBMO_NPOL) stream_collide_npol(s, s->lat[0]);
            else stream_collide_nsol(s, s->lat[0]);
        }
    }
}

/* ---- construction: core::Simulation simulation.cpp:482-519 + setup_domain
 *      domain_initialization.hpp:453-518 --------------------------------------------------- */

plbmo_sim *plbmo_create(int algorithm, int layout, unsigned wg, int scenario, unsigned inner_w, unsigned inner_h,
                        double ivx, double ivy, double irho, double ovx, double ovy, double orho, double tau,
                        int nan_protection, const int8_t *custom_mask)
{
    if (algorithm < 0 || algorithm > 3 || layout < 0 || layout > 2 || wg < 1 || inner_w < 2 || inner_h < 2)
        return NULL;
    plbmo_sim *s = (plbmo_sim *)calloc(1, sizeof(plbmo_sim));
    s->alg = algorithm; s->layout = layout; s->nan_protection = nan_protection;
    s->X = inner_w + 2; s->V = inner_h + 2;
    if (plbmo_domain_for(algorithm, wg, s->X, s->V, &s->dom) != 0) { free(s); return NULL; }
    s->N = s->dom.total_node_count;
    s->Hs = s->dom.horizontal_nodes;
    s->omega = 1 / (real)tau;
    s->rho_out = (real)orho;
    s->flags = (int8_t *)malloc(s->N);
    memset(s->flags, -1, s->N);
    int two = (algorithm == PLBMO_NPTL || algorithm == PLBMO_LPTL);
    s->lat[0] = (real *)malloc(sizeof(real) * 9 * (size_t)s->N);
    s->lat[1] = two ? (real *)malloc(sizeof(real) * 9 * (size_t)s->N) : NULL;
    s->nres = inner_w * inner_h;
    for (int i = 0; i < 4; ++i) s->res[i] = (real *)malloc(sizeof(real) * s->nres);
    for (unsigned i = 0; i < s->nres; ++i) { s->res[0][i] = -1.0; s->res[1][i] = 0; s->res[2][i] = 0; s->res[3][i] = 0; }

    /* set_standstill_values :311-333 */
    real v[9];
    maxwell_boltzmann(0, 0, 1, v);
    for (unsigned n = 0; n < s->N; ++n)
        for (unsigned d = 0; d < 9; ++d) s->lat[0][S_AT(n, d)] = v[d];
    /* set_inout_distribution_values :344-403 */
    real vin[9], vout[9];
    maxwell_boltzmann((real)ivx, (real)ivy, (real)irho, vin);
    maxwell_boltzmann((real)ovx, (real)ovy, (real)orho, vout);
    for (unsigned side = 0; side < 2; ++side)
        for (unsigned j = 0; j + 2 < s->V; ++j) {
            unsigned node = node_index(s, 1 + side * (s->X - 3), 1 + j);
            node = nb(node, side ? 5 : 3, s->Hs);
            for (unsigned d = 0; d < 9; ++d) s->lat[0][S_AT(node, d)] = side ? vout[d] : vin[d];
        }
    if (two) memcpy(s->lat[1], s->lat[0], sizeof(real) * 9 * (size_t)s->N);

    if (scenario == PLBMO_CUSTOM) {
        for (unsigned y = 1; y + 1 < s->V; ++y)
            for (unsigned x = 1; x + 1 < s->X; ++x)
                s->flags[node_index(s, x, y)] = custom_mask ? custom_mask[(x - 1) + (y - 1) * inner_w] : 0;
    } else if (scenario == PLBMO_POROUS) {
        /* porous_medium_mask :265-297 (fresh generator state, as in a new process) */
        plbmo_rand_reset(1);
        for (int y = 2; (unsigned)y < s->V - 2; ++y)
            for (int x = 1; (unsigned)x <= s->X - 2; ++x) {
                int one = 1 + (plbmo_rand() % 10);
                int two_ = 1 + (plbmo_rand() % 10);
                int value = 0;
                if (x % one == one - 1 && y % two_ == two_ - 1) value = 1;
                s->flags[node_index(s, (unsigned)x, (unsigned)y)] = (int8_t)value;
            }
        for (int y = 1; (unsigned)y < s->V; y += (int)(s->V - 3))
            for (int x = 1; (unsigned)x <= s->X - 2; ++x) s->flags[node_index(s, (unsigned)x, (unsigned)y)] = 1;
    } else {
        /* set_pipe_boundaries :214-239 */
        for (unsigned i0 = 0; i0 < 2; ++i0)
            for (unsigned i1 = 0; i1 + 2 < s->X; ++i1)
                s->flags[node_index(s, i1 + 1, i0 * s->V + 1 - 3 * i0)] = 1;
        /* add_stencil :414-440 */
        for (unsigned y = 2; y + 2 < s->V; ++y)
            for (unsigned x = 1; x + 1 < s->X; ++x)
                s->flags[node_index(s, x, y)] = (int8_t)stencil(scenario, x, y, s->V, s->X);
    }
    return s;
}

void plbmo_destroy(plbmo_sim *s)
{
    if (!s) return;
    free(s->flags); free(s->lat[0]); free(s->lat[1]);
    for (int i = 0; i < 4; ++i) free(s->res[i]);
    free(s);
}

void plbmo_results(const plbmo_sim *s, int which, double *out)
{
    for (unsigned i = 0; i < s->nres; ++i) out[i] = (double)s->res[which][i];
}

void plbmo_flags(const plbmo_sim *s, int8_t *out) { memcpy(out, s->flags, s->N); }

size_t plbmo_lattice(const plbmo_sim *s, int which, double *out)
{
    if (!s->lat[which]) return 0;
    size_t n = 9 * (size_t)s->N;
    for (size_t i = 0; i < n; ++i) out[i] = (double)s->lat[which][i];
    return n;
}

void plbmo_get_domain(const plbmo_sim *s, plbmo_domain *out) { *out = s->dom; }

int plbmo_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
