// k_nsol.cu — instantiations of the nsol step kernels (one lattice, in-place AA swap).
#include "plbm_dispatch.cuh"
#include "plbm_launch.h"

namespace plbm {
cudaError_t launch_nsol(int prec, int lay, const StepParams &p, unsigned t, dim3 grid, dim3 block, cudaStream_t s)
{
    if ((t & 1u) == 0) {
        if (lay == COLLISION && block.x == 32 && block.y >= 1 && block.y <= (unsigned)NSOL_STAGE_ROWS) {
            switch (prec) {   // the record layout's even step with its stores staged per block
            case 0: k_nsol_even_staged<0><<<grid, block, 0, s>>>(p); break;
            case 1: k_nsol_even_staged<1><<<grid, block, 0, s>>>(p); break;
            case 2: k_nsol_even_staged<2><<<grid, block, 0, s>>>(p); break;
            case 3: k_nsol_even_staged<3><<<grid, block, 0, s>>>(p); break;
            case 4: k_nsol_even_staged<4><<<grid, block, 0, s>>>(p); break;
            case 5: k_nsol_even_staged<5><<<grid, block, 0, s>>>(p); break;
            case 6: k_nsol_even_staged<6><<<grid, block, 0, s>>>(p); break;
            case 7: k_nsol_even_staged<7><<<grid, block, 0, s>>>(p); break;
            default: return cudaErrorInvalidValue;
            }
            return cudaGetLastError();
        }
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
