// plbm_device.cuh — device-side building blocks shared by every step kernel.
//
// Storage.  Populations live only on the W x H inner nodes of the domain (reference
// coordinates x = 1..X-2, y = 1..V-2, X = W + 2, V = H + 2).  Node n = x' + y' * P with
// x' = x - 1, y' = y - 1 and a row pitch P rounded up to 32 nodes, N = P * H nodes per lattice.
// Ghost nodes are not stored: in the reference they hold constants (standstill weights on the
// bottom/top rows, feq(inlet) on x = 0, feq(outlet) on x = X-1; domain_initialization.hpp:
// 311-403) except the three outlet populations that OutletUpdateKernel rewrites each step
// (non_buffered.hpp:117-129), and those are consumed only by the border node that computed
// them, so the step kernels evaluate the outlet formula in registers instead.
//
// Bounce-back.  EmplaceBounceBackKernel (nptl_kernels.hpp:477-490) copies, for each solid node
// s, S[s][d] = S[s + c_d][8 - d]; a fluid node n pulling direction d from a solid s = n - c_d
// therefore receives its own previous post-collision value S[n][8 - d].  The step kernels read
// that value directly; `links` (one uint16 per node) marks which of the eight pull sources are
// solid (bit d) and whether the node itself is fluid (bit 4).
//
// Layouts (access.hpp:102-172) apply unchanged to the inner grid: collision 9n+d, stream N*d+n,
// bundle 3(d/3)N + d%3 + 3n.
#pragma once
#include <type_traits>

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "plbm_params.h"

namespace plbm {

template <int L>
__device__ __forceinline__ unsigned long long lidx(unsigned long long n, int d, unsigned long long N)
{
    if (L == COLLISION) return 9ull * n + d;
    if (L == STREAM) return N * d + n;
    return 3ull * (d / 3) * N + (d % 3) + 3ull * n;
}

// Index test of the checked build (see STATUS_OUT_OF_RANGE): true when i < n; otherwise records
// the out-of-range index in the status word and returns false so the caller skips the access.
// Without PLBM_CHECKED it is the constant true and costs nothing.
__device__ __forceinline__ bool in_range(unsigned long long i, unsigned long long n, const StepParams &p)
{
#ifdef PLBM_CHECKED
    if (i < n) return true;
    if (p.status) atomicOr(p.status, STATUS_OUT_OF_RANGE);
    return false;
#else
    (void)i; (void)n; (void)p;
    return true;
#endif
}

// Entries of the buffer a population load or store addresses: a lattice or the npol halo.
__device__ __forceinline__ unsigned long long pop_extent(const void *base, const StepParams &p)
{
    return (base == p.halo_in || base == p.halo_out) ? p.halo_elems : p.lat_elems;
}

// links[n], n < N
__device__ __forceinline__ uint16_t link_at(const StepParams &p, unsigned long long n)
{
    return in_range(n, p.N, p) ? p.links[n] : (uint16_t)0;
}

// jy of column W-2 in the previous step, y' < H
__device__ __forceinline__ double jy_prev_at(const StepParams &p, int y)
{
    return in_range((unsigned long long)y, (unsigned long long)p.H, p) ? p.jy_prev[y] : 0.0;
}

// D2Q9 direction d: cx = d % 3 - 1, cy = d / 3 - 1 (access.hpp:203-213).
__device__ __forceinline__ int cxd(int d) { return d % 3 - 1; }
__device__ __forceinline__ int cyd(int d) { return d / 3 - 1; }

// ---- storage types ------------------------------------------------------------------------

template <int PREC> struct Store;
template <> struct Store<F64_STRICT> { using T = double; using C = double; };
template <> struct Store<F64_FAST> { using T = double; using C = double; };
template <> struct Store<F32_REF> { using T = float; using C = float; };
template <> struct Store<F32> { using T = float; using C = float; };
template <> struct Store<F16S> { using T = __half; using C = float; };
template <> struct Store<BF16S> { using T = __nv_bfloat16; using C = float; };
template <> struct Store<F64_Q60> { using T = long long; using C = long long; };
template <> struct Store<F16C> { using T = unsigned short; using C = float; };

// The FP32 / FP16 / BF16 forms hold every population as its deviation from rest,
// df = f - w_d * rho0 (rho0 = 1), in storage AND in the collision: the BGK update is linear in
// the rest part (feq_d - w_d = w_d (drho + 3 cu + 4.5 cu^2 - 1.5 u^2) with rho = 1 + drho), so the
// same arithmetic applied to df yields df'.  Rounding then scales with the deviation from rest,
// not with f itself.
template <int PREC> __host__ __device__ constexpr bool shifted()
{
    return PREC == F32 || PREC == F16S || PREC == BF16S || PREC == F16C;
}

// The 16-bit F16C pattern <-> float (see F16C_DECODE in plbm_params.h).  f16c_bits rounds the
// float32 pattern of v * 2^-110 to 11 significand bits (nearest, ties away from zero: ties are
// one pattern in 2^12) and sets `over` when the magnitude does not fit, |v| >= 0.5 or v NaN (the
// step then reports the status word and the run fails; the pattern itself is not meaningful).
__device__ __forceinline__ float f16c_value(unsigned u)
{
    return __uint_as_float(((u & 0x7FFFu) << 12) | ((u & 0x8000u) << 16)) * F16C_DECODE;
}
__device__ __forceinline__ unsigned f16c_round(unsigned b) { return ((b & 0x7FFFFFFFu) + 0x800u) >> 12; }
__device__ __forceinline__ unsigned f16c_bits(float v, bool &over)
{
    const unsigned b = __float_as_uint(v * F16C_ENCODE);
    const unsigned r = f16c_round(b);
    over = (r & ~F16C_MAX_BITS) != 0;
    return (r & F16C_MAX_BITS) | ((b >> 16) & 0x8000u);
}


template <int PREC>
__device__ __forceinline__ typename Store<PREC>::C ld(const void *base, unsigned long long i, int d, const StepParams &p)
{
    using T = typename Store<PREC>::T;
    const T *b = static_cast<const T *>(base);
    (void)d;
    if (!in_range(i, pop_extent(base, p), p)) return typename Store<PREC>::C(0);
    if constexpr (PREC == F16S) return __half2float(b[i]);   // df * F16_SCALE, the FP16 form's compute value
    else if constexpr (PREC == BF16S) return __bfloat162float(b[i]);
    else if constexpr (PREC == F16C) return f16c_value(b[i]);
    else return b[i];
}

template <int PREC>
__device__ __forceinline__ void st(void *base, unsigned long long i, int d, typename Store<PREC>::C v, const StepParams &p)
{
    using T = typename Store<PREC>::T;
    T *b = static_cast<T *>(base);
    (void)d;
    if (!in_range(i, pop_extent(base, p), p)) return;
    if constexpr (PREC == F16S) b[i] = __float2half_rn(v);
    else if constexpr (PREC == BF16S) b[i] = __float2bfloat16_rn(v);
    else if constexpr (PREC == F16C) {
        bool over;
        b[i] = (unsigned short)f16c_bits(v, over);
        if (over) atomicOr(p.status, 1);
    } else b[i] = v;
}

// ---- the BGK update ------------------------------------------------------------------------

struct Moments { double rho, jx, jy, usq; };
// The float forms keep their moments in float: GB300 issues FP64 at 1/64 of the FP32 rate, so
// they are widened to double only on the steps that write them (observables<PREC>).
struct MomentsF { float rho, jx, jy, usq; };

__device__ __forceinline__ double nan_guard(double v)
{
    // WITH_NAN_PROTECTION (nptl_kernels.hpp:413-432): NaN or > FLT_MAX becomes 0.
    return (isnan(v) || v > 3.4028234663852886e38) ? 0.0 : v;
}

// F64_STRICT: the reference's StreamCollideKernel arithmetic (nptl_kernels.hpp:382-409) in its
// exact IEEE operation order, every operation rounded separately (no contraction).  Terms the
// reference multiplies by a velocity component of 0 or +-1 are exact and are written as the
// sums and negations they reduce to; the results are the same values.
__device__ __forceinline__ Moments collide_f64_strict(double f[9], double omega)
{
    double rho = f[0];
    rho = __dadd_rn(rho, f[1]); rho = __dadd_rn(rho, f[2]); rho = __dadd_rn(rho, f[3]);
    rho = __dadd_rn(rho, f[4]); rho = __dadd_rn(rho, f[5]); rho = __dadd_rn(rho, f[6]);
    rho = __dadd_rn(rho, f[7]); rho = __dadd_rn(rho, f[8]);
    double jx = __dadd_rn(-f[0], f[2]);
    jx = __dsub_rn(jx, f[3]); jx = __dadd_rn(jx, f[5]); jx = __dsub_rn(jx, f[6]); jx = __dadd_rn(jx, f[8]);
    double jy = __dsub_rn(-f[0], f[1]);
    jy = __dsub_rn(jy, f[2]); jy = __dadd_rn(jy, f[6]); jy = __dadd_rn(jy, f[7]); jy = __dadd_rn(jy, f[8]);
    const double usq = __dadd_rn(__dmul_rn(jx, jx), __dmul_rn(jy, jy));
    const double h = __dmul_rn(1.5, usq);
    const double nom = -omega;
    // velocity projections: d0 -(jx+jy), d1 -jy, d2 jx-jy, d3 -jx, d4 0, d5 jx, d6 -(jx-jy), d7 jy, d8 jx+jy
    const double s = __dadd_rn(jx, jy), q = __dsub_rn(jx, jy);
    const double a[4] = { jx, jy, s, q };
    double t3p[4], t3m[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const double c3 = __dmul_rn(3.0, a[k]);
        const double c45 = __dmul_rn(__dmul_rn(4.5, a[k]), a[k]);
        t3p[k] = __dadd_rn(__dadd_rn(rho, c3), c45);   // (rho + 3cu) + 4.5cu^2 with cu = +a
        t3m[k] = __dadd_rn(__dsub_rn(rho, c3), c45);   //                       with cu = -a
    }
    const double w36 = 1.0 / 36, w9 = 1.0 / 9, w49 = 4.0 / 9;
    double feq[9];
    feq[0] = __dmul_rn(w36, __dsub_rn(t3m[2], h));
    feq[1] = __dmul_rn(w9, __dsub_rn(t3m[1], h));
    feq[2] = __dmul_rn(w36, __dsub_rn(t3p[3], h));
    feq[3] = __dmul_rn(w9, __dsub_rn(t3m[0], h));
    feq[4] = __dmul_rn(w49, __dsub_rn(rho, h));
    feq[5] = __dmul_rn(w9, __dsub_rn(t3p[0], h));
    feq[6] = __dmul_rn(w36, __dsub_rn(t3m[3], h));
    feq[7] = __dmul_rn(w9, __dsub_rn(t3p[1], h));
    feq[8] = __dmul_rn(w36, __dsub_rn(t3p[2], h));
#pragma unroll
    for (int d = 0; d < 9; ++d) f[d] = __dadd_rn(__dmul_rn(nom, __dsub_rn(f[d], feq[d])), f[d]);
    return { rho, jx, jy, usq };
}

// F64_FAST: the same BGK update regrouped into 47 FP64 instructions with fused multiply-adds
// (f' = (1-w) f + w feq, feq split into the parts even and odd in the velocity projection).
// Agrees with F64_STRICT to rounding (tested at <= 1e-12 after 10^4 steps).
__device__ __forceinline__ Moments collide_f64_fast(double f[9], double omega)
{
    const double A = f[2] + f[5] + f[8], B = f[0] + f[3] + f[6];
    const double C = f[6] + f[7] + f[8], E = f[0] + f[1] + f[2];
    const double rho = (B + (f[1] + f[4] + f[7])) + A;
    const double jx = A - B, jy = C - E;
    const double usq = fma(jx, jx, jy * jy);
    const double R = fma(-1.5, usq, rho);
    const double om1 = 1.0 - omega;
    const double ow9 = omega * (1.0 / 9), ow36 = omega * (1.0 / 36), ow49 = omega * (4.0 / 9);
    const double b9 = ow9 * R, b36 = ow36 * R;
    f[4] = fma(om1, f[4], ow49 * R);
    // axis pairs (5,3) with u = jx and (7,1) with u = jy; diagonal pairs (8,0) u = jx+jy, (2,6) u = jx-jy
    {
        const double u = jx, sym = fma(4.5 * ow9 * u, u, b9), odd = 3.0 * ow9;
        f[5] = fma(odd, u, fma(om1, f[5], sym));
        f[3] = fma(-odd, u, fma(om1, f[3], sym));
    }
    {
        const double u = jy, sym = fma(4.5 * ow9 * u, u, b9), odd = 3.0 * ow9;
        f[7] = fma(odd, u, fma(om1, f[7], sym));
        f[1] = fma(-odd, u, fma(om1, f[1], sym));
    }
    {
        const double u = jx + jy, sym = fma(4.5 * ow36 * u, u, b36), odd = 3.0 * ow36;
        f[8] = fma(odd, u, fma(om1, f[8], sym));
        f[0] = fma(-odd, u, fma(om1, f[0], sym));
    }
    {
        const double u = jx - jy, sym = fma(4.5 * ow36 * u, u, b36), odd = 3.0 * ow36;
        f[2] = fma(odd, u, fma(om1, f[2], sym));
        f[6] = fma(-odd, u, fma(om1, f[6], sym));
    }
    return { rho, jx, jy, usq };
}

// F32_REF: the reference compiled with USE_FLOAT.  real_type is float, but the literals 9.0/2
// and 3.0/2 are double, so the equilibrium bracket is evaluated in double and rounded to float
// when assigned (nptl_kernels.hpp:401-402); every operation is rounded separately.
__device__ __forceinline__ MomentsF collide_f32_ref(float f[9], float omega)
{
    float rho = f[0];
#pragma unroll
    for (int d = 1; d < 9; ++d) rho = __fadd_rn(rho, f[d]);
    float jx = __fadd_rn(-f[0], f[2]);
    jx = __fsub_rn(jx, f[3]); jx = __fadd_rn(jx, f[5]); jx = __fsub_rn(jx, f[6]); jx = __fadd_rn(jx, f[8]);
    float jy = __fsub_rn(-f[0], f[1]);
    jy = __fsub_rn(jy, f[2]); jy = __fadd_rn(jy, f[6]); jy = __fadd_rn(jy, f[7]); jy = __fadd_rn(jy, f[8]);
    const float usq = __fadd_rn(__fmul_rn(jx, jx), __fmul_rn(jy, jy));
    const double h = __dmul_rn(1.5, (double)usq);
    const float nom = -omega;
    const float s = __fadd_rn(jx, jy), q = __fsub_rn(jx, jy);
    const float a[4] = { jx, jy, s, q };
    double t3p[4], t3m[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float c3 = __fmul_rn(3.0f, a[k]);
        const double c45 = __dmul_rn(__dmul_rn(4.5, (double)a[k]), (double)a[k]);
        t3p[k] = __dadd_rn((double)__fadd_rn(rho, c3), c45);
        t3m[k] = __dadd_rn((double)__fsub_rn(rho, c3), c45);
    }
    const float w36 = (float)(1.0 / 36), w9 = (float)(1.0 / 9), w49 = (float)(4.0 / 9);
    float feq[9];
    feq[0] = (float)__dmul_rn((double)w36, __dsub_rn(t3m[2], h));
    feq[1] = (float)__dmul_rn((double)w9, __dsub_rn(t3m[1], h));
    feq[2] = (float)__dmul_rn((double)w36, __dsub_rn(t3p[3], h));
    feq[3] = (float)__dmul_rn((double)w9, __dsub_rn(t3m[0], h));
    feq[4] = (float)__dmul_rn((double)w49, __dsub_rn((double)rho, h));
    feq[5] = (float)__dmul_rn((double)w9, __dsub_rn(t3p[0], h));
    feq[6] = (float)__dmul_rn((double)w36, __dsub_rn(t3m[3], h));
    feq[7] = (float)__dmul_rn((double)w9, __dsub_rn(t3p[1], h));
    feq[8] = (float)__dmul_rn((double)w36, __dsub_rn(t3p[2], h));
#pragma unroll
    for (int d = 0; d < 9; ++d) f[d] = __fadd_rn(__fmul_rn(nom, __fsub_rn(f[d], feq[d])), f[d]);
    return { rho, jx, jy, usq };
}

// FP32 arithmetic for the F32 / F16S / BF16S storage forms (same regrouping as F64_FAST).  The
// FP16 form collides df * F16_SCALE: the update is linear in f except for the two quadratic
// terms, whose coefficients take qs = 1 / F16_SCALE (qs = 1 for the other forms).
__device__ __forceinline__ MomentsF collide_f32(float f[9], float omega, float qs)
{
    const float A = f[2] + f[5] + f[8], B = f[0] + f[3] + f[6];
    const float C = f[6] + f[7] + f[8], E = f[0] + f[1] + f[2];
    const float rho = (B + (f[1] + f[4] + f[7])) + A;
    const float jx = A - B, jy = C - E;
    const float usq = fmaf(jx, jx, jy * jy);
    const float R = fmaf(-1.5f * qs, usq, rho);
    const float om1 = 1.0f - omega;
    const float ow9 = omega * (1.0f / 9), ow36 = omega * (1.0f / 36), ow49 = omega * (4.0f / 9);
    const float b9 = ow9 * R, b36 = ow36 * R;
    f[4] = fmaf(om1, f[4], ow49 * R);
    { const float u = jx, sym = fmaf(4.5f * ow9 * qs * u, u, b9), odd = 3.0f * ow9;
      f[5] = fmaf(odd, u, fmaf(om1, f[5], sym)); f[3] = fmaf(-odd, u, fmaf(om1, f[3], sym)); }
    { const float u = jy, sym = fmaf(4.5f * ow9 * qs * u, u, b9), odd = 3.0f * ow9;
      f[7] = fmaf(odd, u, fmaf(om1, f[7], sym)); f[1] = fmaf(-odd, u, fmaf(om1, f[1], sym)); }
    { const float u = jx + jy, sym = fmaf(4.5f * ow36 * qs * u, u, b36), odd = 3.0f * ow36;
      f[8] = fmaf(odd, u, fmaf(om1, f[8], sym)); f[0] = fmaf(-odd, u, fmaf(om1, f[0], sym)); }
    { const float u = jx - jy, sym = fmaf(4.5f * ow36 * qs * u, u, b36), odd = 3.0f * ow36;
      f[2] = fmaf(odd, u, fmaf(om1, f[2], sym)); f[6] = fmaf(-odd, u, fmaf(om1, f[6], sym)); }
    return { rho, jx, jy, usq };
}

// ---- F64_Q60: FP64-accuracy populations in 64-bit fixed point ------------------------------
// GB300 issues FP64 at 0.5 T instructions/s but 32-bit integer multiply-adds at ~19 T/s.  The Q60
// form stores each population as round(f * 2^60) in an int64 (Q3.60, resolution 2^-60 ~ 8.7e-19,
// finer than an FP64 ulp of any population >= 2^-7) and performs the BGK update of F64_FAST on the
// integer pipe.  Constants below 1 are held in Q0.64 so a product is the high word of a 64x64
// multiply (within 2 units of 2^-60).  A population leaving [-4, 4) or a momentum leaving [-2, 2)
// sets *status; the host then reports an error.

// High 64 bits of the 128-bit product of unsigned a and b from three 32x32 partial products; the
// dropped low partial product and carries make it at most 2 units low.
__device__ __forceinline__ unsigned long long umulhi_approx(unsigned long long a, unsigned long long b)
{
    const unsigned al = (unsigned)a, ah = (unsigned)(a >> 32), bl = (unsigned)b, bh = (unsigned)(b >> 32);
    return (unsigned long long)ah * bh + __umulhi(ah, bl) + __umulhi(al, bh);
}

// c * v for a constant c in [0, 1) held as round(c * 2^64) and a Q60 value v; result Q60.
__device__ __forceinline__ long long mulc(unsigned long long c, long long v)
{
    const unsigned long long r = umulhi_approx(c, (unsigned long long)v);
    return (long long)(v < 0 ? r - c : r);
}

// a * b for Q60 values with |a|, |b| < 2 (checked by the caller); result Q60.
__device__ __forceinline__ long long mulv(long long a, long long b)
{
    const long long a2 = a << 2, b2 = b << 2;   // Q62
    unsigned long long r = umulhi_approx((unsigned long long)a2, (unsigned long long)b2);
    if (a2 < 0) r -= (unsigned long long)b2;
    if (b2 < 0) r -= (unsigned long long)a2;
    return (long long)r;
}

// Nearest double (ties to even) of v * 2^-60.
__device__ __forceinline__ double q_to_double(long long v)
{
    if (v == 0) return 0.0;
    const unsigned long long sgn = v < 0 ? (1ull << 63) : 0ull;
    const unsigned long long a = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
    const int lz = __clzll((long long)a);
    const unsigned long long n = a << lz;
    unsigned long long mant = n >> 11;
    const unsigned long long rem = n & 0x7FFull;
    mant += (rem > 0x400ull) | ((rem == 0x400ull) & (mant & 1ull));
    // exponent field = 1026 - lz; mant carries the implicit bit (and a rounding carry) into it
    return __longlong_as_double((long long)(sgn | ((((unsigned long long)(1025 - lz)) << 52) + mant)));
}

// v * 2^60 truncated toward zero; |d| < 8.
__device__ __forceinline__ long long double_to_q(double d)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const int e = (int)((b >> 52) & 0x7FF);
    if (e == 0) return 0;
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = e - 1015;
    const long long v = sh >= 0 ? (long long)(m << sh) : (sh <= -64 ? 0 : (long long)(m >> -sh));
    return (b >> 63) ? -v : v;
}

__device__ __forceinline__ unsigned long long q_out_of_range(long long v)
{
    return ((unsigned long long)(v + (1ll << 62))) >> 63;   // 1 unless -4 <= v * 2^-60 < 4
}

// The BGK update of F64_FAST in Q60: f' = f - omega f + omega feq with
// omega feq_d = omega w_d (rho - 1.5 u^2) + 4.5 omega w_d cu^2 + 3 omega w_d cu.  Every constant is
// below 1 for relaxation_time > 0.5 and is applied with mulc; omega f uses omega/2 twice.
__device__ __forceinline__ Moments collide_q60(long long f[9], const StepParams &p)
{
    const long long A = f[2] + f[5] + f[8], B = f[0] + f[3] + f[6];
    const long long C = f[6] + f[7] + f[8], E = f[0] + f[1] + f[2];
    const long long rho = (B + (f[1] + f[4] + f[7])) + A;
    const long long jx = A - B, jy = C - E;
    const long long jx2 = mulv(jx, jx), jy2 = mulv(jy, jy), jxy = mulv(jx, jy);
    const long long usq = jx2 + jy2;
    const long long R = rho - (usq + (usq >> 1));
    const unsigned long long wh = (unsigned long long)p.q_om1;   // omega / 2, Q64
    const long long b9 = mulc((unsigned long long)p.q_ow9, R), b36 = mulc((unsigned long long)p.q_ow36, R);
    f[4] = f[4] + mulc((unsigned long long)p.q_ow49, R) - 2 * mulc(wh, f[4]);
    {
        const long long sym = mulc((unsigned long long)p.q_k9, jx2) + b9, ou = mulc((unsigned long long)p.q_o9, jx);
        f[5] = f[5] + sym + ou - 2 * mulc(wh, f[5]);
        f[3] = f[3] + sym - ou - 2 * mulc(wh, f[3]);
    }
    {
        const long long sym = mulc((unsigned long long)p.q_k9, jy2) + b9, ou = mulc((unsigned long long)p.q_o9, jy);
        f[7] = f[7] + sym + ou - 2 * mulc(wh, f[7]);
        f[1] = f[1] + sym - ou - 2 * mulc(wh, f[1]);
    }
    {
        const long long sym = mulc((unsigned long long)p.q_k36, usq + 2 * jxy) + b36;
        const long long ou = mulc((unsigned long long)p.q_o36, jx + jy);
        f[8] = f[8] + sym + ou - 2 * mulc(wh, f[8]);
        f[0] = f[0] + sym - ou - 2 * mulc(wh, f[0]);
    }
    {
        const long long sym = mulc((unsigned long long)p.q_k36, usq - 2 * jxy) + b36;
        const long long ou = mulc((unsigned long long)p.q_o36, jx - jy);
        f[2] = f[2] + sym + ou - 2 * mulc(wh, f[2]);
        f[6] = f[6] + sym - ou - 2 * mulc(wh, f[6]);
    }
    // populations in [-4, 4) and momenta in [-2, 2), or the status word is set
    unsigned long long bad = (((unsigned long long)(jx + (1ll << 61))) | ((unsigned long long)(jy + (1ll << 61)))) >> 62;
#pragma unroll
    for (int d = 0; d < 9; ++d) bad |= q_out_of_range(f[d]);
    if (bad) atomicOr(p.status, 1);
    // the moments travel as raw fixed-point bits; observables<F64_Q60> converts them when needed
    return { __longlong_as_double(rho), __longlong_as_double(jx), __longlong_as_double(jy), __longlong_as_double(usq) };
}

template <int PREC>
using MomentsOf = typename std::conditional<sizeof(typename Store<PREC>::C) == 4, MomentsF, Moments>::type;

template <int PREC>
__device__ __forceinline__ MomentsOf<PREC> collide(typename Store<PREC>::C f[9], const StepParams &p)
{
    if constexpr (PREC == F64_STRICT) return collide_f64_strict(f, p.omega);
    else if constexpr (PREC == F64_FAST) return collide_f64_fast(f, p.omega);
    else if constexpr (PREC == F32_REF) return collide_f32_ref(f, p.omegaf);
    else if constexpr (PREC == F64_Q60) return collide_q60(f, p);
    else return collide_f32(f, p.omegaf, PREC == F16S ? 1.0f / F16_SCALE : 1.0f);
}

// Outlet populations 0, 3, 6 of a border node (X-2, y), y in [2, V-3], from its other pulled
// values: OutletUpdateKernel non_buffered.hpp:95-129 with f_1 = f[1], f_4 = f[4], f_7 = f[7]
// and f_inverse = {f[8], f[5], f[2]} (the same lattice entries).
template <int PREC>
__device__ __forceinline__ void outlet_fill(typename Store<PREC>::C f[9], double jyo, const StepParams &p)
{
    if constexpr (PREC == F64_STRICT) {
        const double xv = __dadd_rn(-p.rho_out,
                                    __dadd_rn(__dadd_rn(__dadd_rn(f[1], f[4]), f[7]),
                                              __dmul_rn(2.0, __dadd_rn(__dadd_rn(f[8], f[5]), f[2]))));
        const double hd = __dmul_rn(0.5, __dsub_rn(f[1], f[7]));
        const double x6 = __dmul_rn(1.0 / 6, xv), hy = __dmul_rn(0.5, jyo);
        const double g0 = f[8], g1 = f[5], g2 = f[2];
        f[0] = __dsub_rn(__dsub_rn(__dsub_rn(g0, hd), x6), hy);
        f[3] = __dsub_rn(g1, __dmul_rn(2.0 / 3, xv));
        f[6] = __dadd_rn(__dsub_rn(__dadd_rn(g2, hd), x6), hy);
    } else if constexpr (PREC == F64_Q60) {
        const long long xv = -p.q_rho_out + ((f[1] + f[4] + f[7]) + 2 * (f[8] + f[5] + f[2]));
        const long long hd = (f[1] - f[7]) >> 1, x6 = mulc((unsigned long long)p.q_sixth, xv), hy = double_to_q(jyo) >> 1;
        const long long g0 = f[8], g1 = f[5], g2 = f[2];
        f[0] = g0 - hd - x6 - hy;
        f[3] = g1 - mulc((unsigned long long)p.q_two_thirds, xv);
        f[6] = g2 + hd - x6 + hy;
    } else if constexpr (PREC == F32_REF) {
        const float xv = __fadd_rn(-p.rho_outf,
                                   __fadd_rn(__fadd_rn(__fadd_rn(f[1], f[4]), f[7]),
                                             __fmul_rn(2.0f, __fadd_rn(__fadd_rn(f[8], f[5]), f[2]))));
        const double hd = __dmul_rn(0.5, (double)__fsub_rn(f[1], f[7]));
        const double x6 = __dmul_rn(1.0 / 6, (double)xv), hy = __dmul_rn(0.5, jyo);
        const float g0 = f[8], g1 = f[5], g2 = f[2];
        f[0] = (float)__dsub_rn(__dsub_rn(__dsub_rn((double)g0, hd), x6), hy);
        f[3] = (float)__dsub_rn((double)g1, __dmul_rn(2.0 / 3, (double)xv));
        f[6] = (float)__dadd_rn(__dsub_rn(__dadd_rn((double)g2, hd), x6), hy);
    } else {
        using C = typename Store<PREC>::C;
        const C xv = -p.rho_outf + ((f[1] + f[4] + f[7]) + (C)2 * (f[8] + f[5] + f[2]));
        const C hd = (C)0.5 * (f[1] - f[7]), x6 = xv * (C)(1.0 / 6),
                hy = (C)(0.5 * jyo * (PREC == F16S ? (double)F16_SCALE : 1.0));
        const C g0 = f[8], g1 = f[5], g2 = f[2];
        f[0] = g0 - hd - x6 - hy;
        f[3] = g1 - (C)(2.0 / 3) * xv;
        f[6] = g2 + hd - x6 + hy;
    }
}

// Ghost constants in the compute type: rest weights (bottom/top ghost rows), feq(inlet)
// (x = 0), feq(outlet) (x = X-1).
template <int PREC> __device__ __forceinline__ typename Store<PREC>::C g_weight(const StepParams &p, int d)
{
    if constexpr (PREC == F64_Q60) return p.q_weight[d];
    else if constexpr (sizeof(typename Store<PREC>::C) == 8) return p.weight[d]; else return p.weightf[d];
}
template <int PREC> __device__ __forceinline__ typename Store<PREC>::C g_in(const StepParams &p, int d)
{
    if constexpr (PREC == F64_Q60) return p.q_feq_in[d];
    else if constexpr (sizeof(typename Store<PREC>::C) == 8) return p.feq_in[d]; else return p.feq_inf[d];
}
template <int PREC> __device__ __forceinline__ typename Store<PREC>::C g_out(const StepParams &p, int d)
{
    if constexpr (PREC == F64_Q60) return p.q_feq_out[d];
    else if constexpr (sizeof(typename Store<PREC>::C) == 8) return p.feq_out[d]; else return p.feq_outf[d];
}

// Writes the macroscopic observables of node (x', y') when this step is copied to the host,
// and the outlet's jy column every step.
__device__ __forceinline__ void write_observables(const Moments &m, int xi, int yi, const StepParams &p)
{
    double rho = m.rho, jx = m.jx, jy = m.jy;
    if (xi == p.W - 2 && p.jy_next && in_range((unsigned long long)yi, (unsigned long long)p.H, p))
        p.jy_next[yi] = p.nan_protection ? nan_guard(jy) : jy;
    if (p.write_results) {
        double ja = sqrt(m.usq);
        if (p.nan_protection) { rho = nan_guard(rho); jx = nan_guard(jx); jy = nan_guard(jy); ja = nan_guard(ja); }
        const unsigned long long r = (unsigned long long)xi + (unsigned long long)yi * p.W;
        if (!in_range(r, (unsigned long long)p.W * p.H, p)) return;
        p.rho[r] = rho; p.jx[r] = jx; p.jy[r] = jy; p.jabs[r] = ja;
    }
}

// Float results are sqrt'ed in float in the USE_FLOAT build (sycl::sqrt on real_type).
__device__ __forceinline__ void write_observables_f32ref(const Moments &m, int xi, int yi, const StepParams &p)
{
    double rho = m.rho, jx = m.jx, jy = m.jy;
    if (xi == p.W - 2 && p.jy_next && in_range((unsigned long long)yi, (unsigned long long)p.H, p))
        p.jy_next[yi] = p.nan_protection ? nan_guard(jy) : jy;
    if (p.write_results) {
        double ja = (double)sqrtf((float)m.usq);
        if (p.nan_protection) { rho = nan_guard(rho); jx = nan_guard(jx); jy = nan_guard(jy); ja = nan_guard(ja); }
        const unsigned long long r = (unsigned long long)xi + (unsigned long long)yi * p.W;
        if (!in_range(r, (unsigned long long)p.W * p.H, p)) return;
        p.rho[r] = rho; p.jx[r] = jx; p.jy[r] = jy; p.jabs[r] = ja;
    }
}

template <int PREC>
__device__ __forceinline__ void observables(const MomentsOf<PREC> &m, int xi, int yi, const StepParams &p)
{
    if (!p.write_results && xi != p.W - 2) return;   // nothing is written on this step
    if constexpr (PREC == F32_REF) {
        const Moments d = { (double)m.rho, (double)m.jx, (double)m.jy, (double)m.usq };
        write_observables_f32ref(d, xi, yi, p);
    } else if constexpr (PREC == F64_Q60) {
        const Moments d = { q_to_double(__double_as_longlong(m.rho)), q_to_double(__double_as_longlong(m.jx)),
                            q_to_double(__double_as_longlong(m.jy)), q_to_double(__double_as_longlong(m.usq)) };
        write_observables(d, xi, yi, p);
    } else if constexpr (shifted<PREC>()) {
        // rho = rho0(x') + drho; the FP16 form's moments carry F16_SCALE
        const double us = PREC == F16S ? 1.0 / F16_SCALE : 1.0;
        const Moments d = { (p.shift_a - p.shift_g * xi) + (double)m.rho * us, (double)m.jx * us, (double)m.jy * us,
                            (double)m.usq * us * us };
        write_observables(d, xi, yi, p);
    } else {
        write_observables(m, xi, yi, p);
    }
}

// True when node (x', y') is an outlet border node whose 0/3/6 populations come from the
// density-outlet formula (reference x = X-2, y in [2, V-3]).
__device__ __forceinline__ bool is_outlet_row(int xi, int yi, const StepParams &p)
{
    return p.outlet_mode == 0 && xi == p.W - 1 && yi >= 1 && yi <= p.H - 2;
}

}  // namespace plbm
