// omx_kernels_fast.cu -- FP32 fused path of the Yee/CPML/ADE half-step kernels.  FP32 field
// state with FP64-precomputed coefficients rounded once to FP32; multiply-adds contract to FMA.
#include <cuda_runtime.h>
#include "omx_fused2d.cuh"

namespace omx {

template <> void launch_h<float>(const FieldPtrs<float> &F, const GridArgs<float> &G, void *s)
{
    launch_h_impl<float, false>(F, G, s);
}
template <> void launch_e<float>(const FieldPtrs<float> &F, const GridArgs<float> &G, void *s)
{
    launch_e_impl<float, false>(F, G, s);
}

void launch_fused_tmz(const Fused2Args &A, const GridArgs<float> &G, void *s)
{
    constexpr int JCH = 32;
    const int threads = G.L.nx / 4;
    dim3 b(128, 1, 1), g((threads + 127) / 128, (G.L.ny + JCH - 1) / JCH, 1);
    if (A.psi_ezx) k_fused_tmz<JCH, true><<<g, b, 0, (cudaStream_t)s>>>(A, G);
    else k_fused_tmz<JCH, false><<<g, b, 0, (cudaStream_t)s>>>(A, G);
}

void launch_ade_post(const FieldPtrs<float> &Fin, const FieldPtrs<float> &Fout, const GridArgs<float> &G, void *s)
{
    if (G.ade_n <= 0) return;
    k_ade_post<<<(G.ade_n + 127) / 128, 128, 0, (cudaStream_t)s>>>(Fin, Fout, G);
}

}  // namespace omx
