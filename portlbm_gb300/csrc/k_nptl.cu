// k_nptl.cu — instantiations of the nptl step kernel (two lattices, 2-D blocks).
#include "plbm_dispatch.cuh"
#include "plbm_launch.h"

namespace plbm {
cudaError_t launch_nptl(int prec, int lay, const StepParams &p, dim3 grid, dim3 block, cudaStream_t s, bool porous)
{
    const bool two_byte = prec == F16S || prec == BF16S || prec == F16C;
    const dim3 vb(32, VEC_ROWS), vg((unsigned)((p.P + 32 * VEC - 1) / (32 * VEC)), (unsigned)((p.H + VEC_ROWS - 1) / VEC_ROWS));
    // 2-byte storage in the stream layout on porous geometries: vectorised rows with the bounce-back
    // merged word-wise
    if (porous && two_byte && lay == STREAM) {
        if (prec == F16S) k_nptl_vec_porous<F16S><<<vg, vb, 0, s>>>(p);
        else if (prec == F16C) k_nptl_vec_porous<F16C><<<vg, vb, 0, s>>>(p);
        else k_nptl_vec_porous<BF16S><<<vg, vb, 0, s>>>(p);
        return cudaGetLastError();
    }
    if (porous && ((prec >= F32 && prec <= BF16S) || prec == F16C)) {
        switch (prec * 3 + lay) {
            PLBM_POROUS_CASES(k_nptl)
        default: return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    }
    // 2-byte storage in the stream layout: vectorised rows (launch shape of its own)
    if (two_byte && lay == STREAM) {
        if (prec == F16S) k_nptl_vec<F16S><<<vg, vb, 0, s>>>(p);
        else if (prec == F16C) k_nptl_vec<F16C><<<vg, vb, 0, s>>>(p);
        else k_nptl_vec<BF16S><<<vg, vb, 0, s>>>(p);
        return cudaGetLastError();
    }
    switch (prec * 3 + lay) {
        PLBM_ALL_CASES(k_nptl)
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
}  // namespace plbm
