// k_nptl.cu — instantiations of the nptl step kernel (two lattices, 2-D blocks).
#include "plbm_dispatch.cuh"
#include "plbm_launch.h"

namespace plbm {
cudaError_t launch_nptl(int prec, int lay, const StepParams &p, dim3 grid, dim3 block, cudaStream_t s)
{
    switch (prec * 3 + lay) {
        PLBM_ALL_CASES(k_nptl)
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
}  // namespace plbm
