// omx_kernels_fast.cu -- FP32 fused path of the Yee/CPML/ADE half-step kernels.  FP32 field
// state with FP64-precomputed coefficients rounded once to FP32; multiply-adds contract to FMA.
#include <cuda_runtime.h>

#include <algorithm>
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

static int persistent_blocks(const void *kernel)
{
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, 0);
    return (sms > 0 ? sms : 152) * (per_sm > 0 ? per_sm : 1);
}

void launch_fused_tmz(const Fused2Args &A, const GridArgs<float> &G, void *s)
{
    const int nstrip = (G.L.nx / 4 + 127) / 128;
    const void *k = A.psi_ezx ? (const void *)k_fused_tmz<true> : (const void *)k_fused_tmz<false>;
    static int blocks_true = 0, blocks_false = 0;
    int &nb = A.psi_ezx ? blocks_true : blocks_false;
    if (nb == 0) nb = persistent_blocks(k);
    const long long rows = (long long)nstrip * G.L.ny;
    const int grid = (int)std::min<long long>(nb, rows);
    if (A.psi_ezx) k_fused_tmz<true><<<grid, 128, 0, (cudaStream_t)s>>>(A, G, nstrip);
    else k_fused_tmz<false><<<grid, 128, 0, (cudaStream_t)s>>>(A, G, nstrip);
}

void launch_ade_post(const FieldPtrs<float> &Fin, const FieldPtrs<float> &Fout, const GridArgs<float> &G, void *s)
{
    if (G.ade_n <= 0) return;
    k_ade_post<<<(G.ade_n + 127) / 128, 128, 0, (cudaStream_t)s>>>(Fin, Fout, G);
}

}  // namespace omx
