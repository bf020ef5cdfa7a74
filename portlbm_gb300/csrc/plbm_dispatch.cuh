// plbm_dispatch.cuh — maps runtime (precision, layout) to a template instantiation.
#pragma once
#include "plbm_kernels.cuh"

#define PLBM_CASE(KER, PR, LA) case (PR) * 3 + (LA): KER<PR, LA><<<grid, block, 0, s>>>(p); break;
#define PLBM_ALL_CASES(KER)                                                                   \
    PLBM_CASE(KER, 0, 0) PLBM_CASE(KER, 0, 1) PLBM_CASE(KER, 0, 2)                             \
    PLBM_CASE(KER, 1, 0) PLBM_CASE(KER, 1, 1) PLBM_CASE(KER, 1, 2)                             \
    PLBM_CASE(KER, 2, 0) PLBM_CASE(KER, 2, 1) PLBM_CASE(KER, 2, 2)                             \
    PLBM_CASE(KER, 3, 0) PLBM_CASE(KER, 3, 1) PLBM_CASE(KER, 3, 2)                             \
    PLBM_CASE(KER, 4, 0) PLBM_CASE(KER, 4, 1) PLBM_CASE(KER, 4, 2)                             \
    PLBM_CASE(KER, 5, 0) PLBM_CASE(KER, 5, 1) PLBM_CASE(KER, 5, 2)                             \
    PLBM_CASE(KER, 6, 0) PLBM_CASE(KER, 6, 1) PLBM_CASE(KER, 6, 2)                             \
    PLBM_CASE(KER, 7, 0) PLBM_CASE(KER, 7, 1) PLBM_CASE(KER, 7, 2)

// The porous gather of the shifted forms (f32, f16s, bf16s, f16c; the unshifted forms have one gather).
#define PLBM_POROUS_CASE(KER, PR, LA) case (PR) * 3 + (LA): KER<PR, LA, true><<<grid, block, 0, s>>>(p); break;
#define PLBM_POROUS_CASES(KER)                                                                \
    PLBM_POROUS_CASE(KER, 3, 0) PLBM_POROUS_CASE(KER, 3, 1) PLBM_POROUS_CASE(KER, 3, 2)        \
    PLBM_POROUS_CASE(KER, 4, 0) PLBM_POROUS_CASE(KER, 4, 1) PLBM_POROUS_CASE(KER, 4, 2)        \
    PLBM_POROUS_CASE(KER, 5, 0) PLBM_POROUS_CASE(KER, 5, 1) PLBM_POROUS_CASE(KER, 5, 2)        \
    PLBM_POROUS_CASE(KER, 7, 0) PLBM_POROUS_CASE(KER, 7, 1) PLBM_POROUS_CASE(KER, 7, 2)
