// k_nsol.cu — instantiations of the nsol step kernels (one lattice, in-place AA swap).
#include "plbm_dispatch.cuh"
#include "plbm_launch.h"

namespace plbm {
cudaError_t launch_nsol(int prec, int lay, const StepParams &p, unsigned t, dim3 grid, dim3 block, cudaStream_t s)
{
    if ((t & 1u) == 0) {
        switch (prec * 3 + lay) {
            PLBM_ALL_CASES(k_nsol_even)
        default: return cudaErrorInvalidValue;
        }
    } else {
        switch (prec * 3 + lay) {
            PLBM_ALL_CASES(k_nsol_odd)
        default: return cudaErrorInvalidValue;
        }
    }
    return cudaGetLastError();
}
}  // namespace plbm
