// plbm_power.h — core::power_functions (include/lbm/core/simulation.hpp:373-446): which power of
// 4 / of 2 a work-group size is (0 when it is none), with the reference's own tests, which the
// Domain tile shape and the benchmark's work-group sweep both depend on.
#pragma once

#include <cstddef>

namespace plbm {

inline size_t which_power_of_4(size_t x)
{
    size_t checkbit = 3, pow = 0;
    if ((x & 0x1) || x == 0) return 0;
    while (!(checkbit & x)) { x >>= 2; pow++; }
    return !(x & 2) ? pow : 0;
}

inline size_t which_power_of_2(size_t x)
{
    size_t checkbit = 1, pow = 0;
    if ((x & 0x1) || x == 0) return 0;
    while (!(checkbit & x)) { x >>= 1; pow++; }
    return !(x >> 1 | 0) ? pow : 0;
}

}  // namespace plbm
