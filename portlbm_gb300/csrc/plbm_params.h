// plbm_params.h — step parameters shared by host and device code (host-safe header).
#pragma once

#include <stdint.h>

namespace plbm {

enum Layout { COLLISION = 0, STREAM = 1, BUNDLE = 2 };
enum Precision { F64_STRICT = 0, F64_FAST = 1, F32_REF = 2, F32 = 3, F16S = 4, BF16S = 5, F64_Q60 = 6, F16C = 7 };

constexpr uint16_t LINK_FLUID = 1u << 4;
// Set by k_links on the nodes of the first and last inner row and column: with it, an interior
// fluid node whose eight sources are fluid is exactly links == LINK_FLUID.
constexpr uint16_t LINK_EDGE = 1u << 9;

// FP16 storage holds df * 2^12: deviations down to ~1.5e-8 stay in half's normal range (min
// normal 6.1e-5) while the largest deviations of a stable run (|df| < 1) stay far below its
// maximum, 65504.  The FP16 form also computes on these scaled values (its constants are scaled
// the same way), so loads and stores need no rescaling.
constexpr float F16_SCALE = 4096.0f;

// F16C storage: the deviation df in a 16-bit float of 1 sign, 4 exponent and 11 significand bits
// (the layout of a float32 with its exponent limited to 0..15 and its significand cut to 11 bits),
// scaled so that |df| < 0.5 is representable: normal values from 2^-16, gradual underflow below
// with a resolution of 2^-27.  IEEE half spends 5 exponent bits on a range the deviations never
// use; this form gives that bit to the significand (relative rounding 2^-12 instead of 2^-11).
// Decoding places the 15 magnitude bits in a float32 pattern and multiplies by 2^110; encoding
// multiplies by 2^-110 and rounds the pattern to 11 significand bits (nearest, ties away from zero).
constexpr float F16C_DECODE = 1.2980742146337069e33f;   // 2^110
constexpr float F16C_ENCODE = 7.7037197775489434e-34f;  // 2^-110
constexpr unsigned F16C_MAX_BITS = 0x7FFFu;            // largest magnitude pattern: (2 - 2^-11) * 2^-2

// The checked build (compiled with -DPLBM_CHECKED, libplbm_checked.so) compares every lattice,
// link, result, jy-column and halo index of the step kernels with its buffer's extent; an index
// outside it sets this bit of the status word and the access is skipped (no trap).  The host turns
// the bit into PLBM_ERR_CUDA after the steps.
constexpr int STATUS_OUT_OF_RANGE = 0x100;
#ifdef PLBM_CHECKED
constexpr bool CHECKED_BUILD = true;
#else
constexpr bool CHECKED_BUILD = false;
#endif

// Nodes per thread of the two-lattice kernels (nptl rows, lptl grid strides), per precision.
constexpr int rows_per_thread(int) { return 1; }

// Step parameters, passed by value to every step kernel.
struct StepParams {
    void *lat0;                 // source lattice (two-lattice) / the lattice (one-lattice)
    void *lat1;                 // destination lattice (two-lattice only)
    const uint16_t *links;      // per node: bit d (d != 4) pull source solid, bit 4 fluid
    double *rho, *jx, *jy, *jabs;   // results, W*H doubles, row-major over the inner domain
    const double *jy_prev;      // jy of the previous step at x' = W-2 (H entries)
    double *jy_next;            // jy of this step at x' = W-2
    double *halo_in, *halo_out; // one-lattice tile halos (npol) [cols | rows]
    int W, H, P;
    unsigned long long N;
    int tile_w, tile_h;         // npol tile
    int n_col_bounds, n_row_bounds;
    double omega;               // 1 / relaxation_time, in the storage precision's value
    double rho_out;
    double feq_in[9], feq_out[9], weight[9];   // ghost constants in the policy's arithmetic
    // float copies for the FP32-arithmetic forms (a double->float conversion in the inner loop
    // would run on the FP64 pipe)
    float feq_inf[9], feq_outf[9], weightf[9];
    float omegaf, rho_outf;
    // Shifted forms (F32, F16S, BF16S) hold f_d - w_d * rho0(x') with rho0(x') = shift_a - shift_g * x'.
    // Two-lattice pull schemes use the straight profile between the inlet ghost column (x' = -1,
    // rho_in) and the outlet ghost column (x' = W, rho_out); the others use rho0 = 1.  Every
    // constant above is then relative to the rho0 of the node that reads it; a value pulled from
    // column x' - cx_d is re-referenced by adding shift_cx[d] = w_d * shift_g * cx_d, and a wall
    // ghost (rest state, rho = 1) reads weightf[d] + shift_wg[d] * x' = w_d (1 - rho0(x')).
    double shift_a, shift_g;
    float shift_wg[9], shift_cx[9];
    // F64_Q60: 64-bit fixed-point constants (value * 2^60, rounded from the double constants) and
    // the device word that records a population leaving the fixed-point range
    long long q_weight[9], q_feq_in[9], q_feq_out[9];
    long long q_om1, q_ow49, q_ow9, q_ow36, q_k9, q_k36, q_o9, q_o36, q_rho_out, q_sixth, q_two_thirds;
    int *status;                // F64_Q60 / F16C: bit 0 when a value leaves the storage range;
                                // checked builds: STATUS_OUT_OF_RANGE when an index leaves its buffer
    // Buffer extents (entries) for the checked build's index tests: each lattice, the npol halo.
    unsigned long long lat_elems, halo_elems;
    int outlet_mode;            // 0: Zou/He-type density outlet; 1: constant feq(outlet) ghost
    int nan_protection;
    int write_results;          // this step is copied to the host
};

}  // namespace plbm
