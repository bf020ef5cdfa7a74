// k_lptl.cu — instantiations of the lptl step kernel (two lattices, 1-D launch).
#include "plbm_dispatch.cuh"
#include "plbm_launch.h"

namespace plbm {
cudaError_t launch_lptl(int prec, int lay, const StepParams &p, dim3 grid, dim3 block, cudaStream_t s, bool porous)
{
    if (porous && ((prec >= F32 && prec <= BF16S) || prec == F16C)) {
        switch (prec * 3 + lay) {
            PLBM_POROUS_CASES(k_lptl)
        default: return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    }
    switch (prec * 3 + lay) {
        PLBM_ALL_CASES(k_lptl)
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
}  // namespace plbm
