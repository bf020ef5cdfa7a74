// plbm_consts.h — host-side constants shared by the handler and the batch code: the rest and
// boundary equilibria (maxwell_boltzmann_distribution, include/lbm/core/simulation.hpp:333-350)
// and the fixed-point constants of the F64_Q60 form, so both paths derive them identically.
#pragma once

#include <cmath>

#include "plbm_params.h"

namespace plbm {

// round(x * 2^60) for populations (Q3.60).
inline long long q60(long double x) { return (long long)std::llroundl(x * 1152921504606846976.0L); }

// round(c * 2^64) for constants 0 <= c < 1 (Q0.64), returned as the unsigned bit pattern.
inline long long q64(long double c)
{
    const long double v = c * 18446744073709551616.0L + 0.5L;
    const unsigned long long u = v >= 18446744073709551615.0L ? 18446744073709551615ull : (unsigned long long)v;
    return (long long)u;
}

// maxwell_boltzmann_distribution in real_type R (std::pow(v, 2) promotes to double).
template <typename R>
inline void maxwell_boltzmann(R ux, R uy, R rho, R *t)
{
    static const R W[9] = { (R)(1.0 / 36), (R)(1.0 / 9), (R)(1.0 / 36), (R)(1.0 / 9), (R)(4.0 / 9),
                            (R)(1.0 / 9), (R)(1.0 / 36), (R)(1.0 / 9), (R)(1.0 / 36) };
    for (int d = 0; d < 9; ++d) {
        const int vx = (d % 3) - 1, vy = (d / 3) - 1;
        t[d] = (R)(W[d] * (rho + 3 * (vx * ux + vy * uy) + 9.0 / 2 * std::pow((double)(vx * ux + vy * uy), 2) -
                           3.0 / 2 * (ux * ux + uy * uy)));
    }
}

// Fixed-point constants from the double constants the reference computes with (1/tau, w_d,
// 1.0/6, 2.0/3), evaluated in long double; needs b.omega, b.rho_out, b.weight/feq_in/feq_out.
inline void fill_q60_constants(StepParams &b)
{
    const long double om = (long double)b.omega, w9 = 1.0 / 9, w36 = 1.0 / 36, w49 = 4.0 / 9;
    b.q_om1 = q64(om / 2);   // the Q60 kernel applies omega as twice omega/2
    b.q_ow49 = q64(om * w49);
    b.q_ow9 = q64(om * w9);
    b.q_ow36 = q64(om * w36);
    b.q_k9 = q64(4.5L * om * w9);
    b.q_k36 = q64(4.5L * om * w36);
    b.q_o9 = q64(3.0L * om * w9);
    b.q_o36 = q64(3.0L * om * w36);
    b.q_rho_out = q60((long double)b.rho_out);
    b.q_sixth = q64((long double)(1.0 / 6));
    b.q_two_thirds = q64((long double)(2.0 / 3));
    for (int d = 0; d < 9; ++d) {
        b.q_weight[d] = q60((long double)b.weight[d]);
        b.q_feq_in[d] = q60((long double)b.feq_in[d]);
        b.q_feq_out[d] = q60((long double)b.feq_out[d]);
    }
}

// Float constants of the FP32-arithmetic forms, rounded once from the double constants
// (b.W, b.weight, b.feq_in, b.feq_out, b.rho_out, b.omega must be set).  For the shifted forms
// the reference density is rho0(x') = a - g x' (see StepParams): profile = true gives the straight
// inlet-outlet profile a = rho_in - g, g = (rho_in - rho_out) / (W + 1); otherwise rho0 = 1.
// `scale` multiplies the shifted constants (F16_SCALE for the FP16 form, which computes on
// scaled values).
inline void fill_float_constants(StepParams &b, bool shifted, bool profile, double rho_in, double rho_out,
                                 double scale = 1.0)
{
    const double g = shifted && profile ? (rho_in - rho_out) / (b.W + 1) : 0.0;
    const double a = shifted && profile ? rho_in - g : 1.0;
    b.shift_a = a;
    b.shift_g = g;
    const double r_in = a, r_out = a - g * (b.W - 1);   // rho0 of the columns that read the inlet / outlet ghosts
    for (int d = 0; d < 9; ++d) {
        const double w = b.weight[d];
        const int cx = d % 3 - 1;
        b.weightf[d] = shifted ? (float)(w * (1.0 - a) * scale) : (float)w;
        b.feq_inf[d] = shifted ? (float)((b.feq_in[d] - w * r_in) * scale) : (float)b.feq_in[d];
        b.feq_outf[d] = shifted ? (float)((b.feq_out[d] - w * r_out) * scale) : (float)b.feq_out[d];
        b.shift_wg[d] = (float)(w * g * scale);
        b.shift_cx[d] = (float)(w * g * cx * scale);
    }
    b.omegaf = (float)b.omega;
    // outlet: f1+f4+f7+2(f8+f5+f2) carries exactly 1 in rest weights, so xv = (rho0 - rho_out) + sum(df)
    b.rho_outf = shifted ? (float)((b.rho_out - r_out) * scale) : (float)b.rho_out;
}

}  // namespace plbm
