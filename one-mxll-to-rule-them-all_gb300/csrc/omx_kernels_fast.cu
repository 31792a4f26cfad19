// omx_kernels_fast.cu -- FP32 fused path of the Yee/CPML/ADE half-step kernels.  FP32 field
// state with FP64-precomputed coefficients rounded once to FP32; multiply-adds contract to FMA.
#include <cuda_runtime.h>
#include "omx_stencil.cuh"

namespace omx {

template <> void launch_h<float>(const FieldPtrs<float> &F, const GridArgs<float> &G, void *s)
{
    launch_h_impl<float, false>(F, G, s);
}
template <> void launch_e<float>(const FieldPtrs<float> &F, const GridArgs<float> &G, void *s)
{
    launch_e_impl<float, false>(F, G, s);
}

}  // namespace omx
