// k_npol.cu — instantiations of the npol step kernel (one lattice in place, tile halos).
#include "plbm_dispatch.cuh"
#include "plbm_launch.h"

namespace plbm {
cudaError_t launch_npol(int prec, int lay, const StepParams &p, dim3 grid, dim3 block, cudaStream_t s)
{
    switch (prec * 3 + lay) {
        PLBM_ALL_CASES(k_npol)
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
}  // namespace plbm
