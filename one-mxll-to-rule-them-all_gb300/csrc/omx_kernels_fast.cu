// omx_kernels_fast.cu -- FP32 fused path of the Yee/CPML/ADE half-step kernels.  FP32 field
// state with FP64-precomputed coefficients rounded once to FP32; multiply-adds contract to FMA.
#include <cuda_runtime.h>

#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include "omx_batch.cuh"
#include "omx_fused2d.cuh"
#include "omx_fused3d.cuh"

namespace omx {

template <> void launch_h<float>(const FieldPtrs<float> &F, const GridArgs<float> &G, void *s)
{
    launch_h_impl<float, false>(F, G, s);
}
template <> void launch_e<float>(const FieldPtrs<float> &F, const GridArgs<float> &G, void *s)
{
    launch_e_impl<float, false>(F, G, s);
}

static int persistent_blocks(const void *kernel, size_t smem, int threads = 128)
{
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
    return (sms > 0 ? sms : 152) * (per_sm > 0 ? per_sm : 1);
}

// Fused-kernel forms: "regs" (register prefetch of the next row), "tmaD" (rows staged by bulk
// copies into a D-slot shared-memory ring, one block barrier per row) and "wsD" (the same ring
// filled by a dedicated copy warp, full / empty barriers per slot).  The default is ws4, the
// fastest on the 4096^2 TMz workload; OMX_FUSED_KERNEL overrides it for the process and
// omx_autotune picks a form per grid.
static int default_fused_form()
{
    static int form = -1;
    if (form < 0) {
        form = 44;   // ws4w8: eight compute warps, 4-slot ring (measured fastest on 4096^2)
        if (const char *v = getenv("OMX_FUSED_KERNEL")) {
            if (!strcmp(v, "regs")) form = 0;
            else if (!strcmp(v, "tma4")) form = 4;
            else if (!strcmp(v, "tma5")) form = 5;
            else if (!strcmp(v, "tma6")) form = 6;
            else if (!strcmp(v, "tma8")) form = 8;
            else if (!strcmp(v, "ws4")) form = 14;
            else if (!strcmp(v, "ws5")) form = 15;
            else if (!strcmp(v, "ws6")) form = 16;
            else if (!strcmp(v, "ws4x2")) form = 24;
            else if (!strcmp(v, "ws5x2")) form = 25;
            else if (!strcmp(v, "ws4w8")) form = 44;
            else if (!strcmp(v, "ws5w8")) form = 45;
            else if (!strcmp(v, "rt4")) form = 34;
            else if (!strcmp(v, "rt6")) form = 36;
        }
    }
    return form;
}

constexpr int FZ_MAX_DEV = 64;

template <bool X, int D> static void launch_tma(const Fused2Args &A, const GridArgs<float> &G, int nstrip, cudaStream_t s)
{
    const size_t smem = D * sizeof(FzStage) + D * sizeof(uint64_t);
    static int nb[FZ_MAX_DEV] = {};       // persistent grid per device (the smem opt-in is per device)
    int dev = 0;
    cudaGetDevice(&dev);
    int &n = nb[dev < FZ_MAX_DEV ? dev : 0];
    if (n == 0) {
        cudaFuncSetAttribute(k_fused_tmz_tma<X, D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        n = persistent_blocks((const void *)k_fused_tmz_tma<X, D>, smem);
    }
    const int grid = (int)std::min<long long>(n, (long long)nstrip * G.L.ny);
    k_fused_tmz_tma<X, D><<<grid, 128, smem, s>>>(A, G, nstrip);
}

template <bool X, int D, int CH, int NW = 4>
static void launch_ws(const Fused2Args &A, const GridArgs<float> &G, cudaStream_t s)
{
    constexpr int SW = NW * CH / 4;   // stage width in units of 512 columns
    const size_t smem = D * sizeof(FzStageT<SW>) + 2 * D * sizeof(uint64_t);
    const int cols = 32 * NW * CH;    // float4 groups per strip
    const int nstrip = (G.L.nx / 4 + cols - 1) / cols;
    static int nb[FZ_MAX_DEV] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    int &n = nb[dev < FZ_MAX_DEV ? dev : 0];
    if (n == 0) {
        cudaFuncSetAttribute(k_fused_tmz_ws<X, D, CH, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        n = persistent_blocks((const void *)k_fused_tmz_ws<X, D, CH, NW>, smem, 32 * (NW + 1));
    }
    const int grid = (int)std::min<long long>(n, (long long)nstrip * G.L.ny);
    k_fused_tmz_ws<X, D, CH, NW><<<grid, 32 * (NW + 1), smem, s>>>(A, G, nstrip);
}

template <bool X, int R> static void launch_rt(const Fused2Args &A, const GridArgs<float> &G, int nstrip, cudaStream_t s)
{
    const int ntile = (G.L.ny + R - 1) / R;
    k_fused_tmz_rt<X, R><<<(unsigned)(nstrip * ntile), 128, 0, s>>>(A, G, ntile);
}

template <bool X> static void launch_regs(const Fused2Args &A, const GridArgs<float> &G, int nstrip, cudaStream_t s)
{
    static int nb[FZ_MAX_DEV] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    int &n = nb[dev < FZ_MAX_DEV ? dev : 0];
    if (n == 0) n = persistent_blocks((const void *)k_fused_tmz<X>, 0);
    const int grid = (int)std::min<long long>(n, (long long)nstrip * G.L.ny);
    k_fused_tmz<X><<<grid, 128, 0, s>>>(A, G, nstrip);
}

template <bool X>
static void launch_form(const Fused2Args &A, const GridArgs<float> &G, int form, int nstrip, cudaStream_t s)
{
    switch (form >= 0 ? form : default_fused_form()) {
    case 0: launch_regs<X>(A, G, nstrip, s); break;
    case 4: launch_tma<X, 4>(A, G, nstrip, s); break;
    case 6: launch_tma<X, 6>(A, G, nstrip, s); break;
    case 8: launch_tma<X, 8>(A, G, nstrip, s); break;
    case 16: launch_ws<X, 6, 1>(A, G, s); break;
    case 5: launch_tma<X, 5>(A, G, nstrip, s); break;
    case 15: launch_ws<X, 5, 1>(A, G, s); break;
    case 24: launch_ws<X, 4, 2>(A, G, s); break;
    case 44: launch_ws<X, 4, 1, 8>(A, G, s); break;
    case 45: launch_ws<X, 5, 1, 8>(A, G, s); break;
    case 34: launch_rt<X, 4>(A, G, nstrip, s); break;
    case 36: launch_rt<X, 6>(A, G, nstrip, s); break;
    case 25: launch_ws<X, 5, 2>(A, G, s); break;
    case 14: launch_ws<X, 4, 1>(A, G, s); break;
    default: launch_ws<X, 4, 1, 8>(A, G, s); break;
    }
}

void launch_fused_tmz(const Fused2Args &A, const GridArgs<float> &G, int form, void *s)
{
    const int nstrip = (G.L.nx / 4 + 127) / 128;
    if (A.psi_ezx) launch_form<true>(A, G, form, nstrip, (cudaStream_t)s);
    else launch_form<false>(A, G, form, nstrip, (cudaStream_t)s);
}

void launch_fused3(const Fused3Args &A, const GridArgs<float> &G, int kch, void *s)
{
    const int m = kch > 0 ? kch : 16;
    const dim3 b(32, F3_BY, 1), g((unsigned)((G.L.nx + 31) / 32), (unsigned)((G.L.ny + F3_BY - 1) / F3_BY),
                                  (unsigned)((G.L.nz + m - 1) / m));
    k_fused3<<<g, b, 0, (cudaStream_t)s>>>(A, G, m);
}

template <> void launch_batch3<float>(int pass, const BatchGrid<float> *g, int n, long long total, int kch,
                                     int blocks, void *s)
{
    launch_batch3_impl<float, false>(pass, g, n, total, kch, blocks, s);
}
template <> int batch3_blocks<float>() { return batch3_blocks_impl<float, false>(); }
template <> void launch_ade<float>(const FieldPtrs<float> &F, const GridArgs<float> &G, void *s)
{
    if (G.ade_n > 0) k_ade<float><<<(G.ade_n + 127) / 128, 128, 0, (cudaStream_t)s>>>(F, G);
}

void launch_ade_post(const FieldPtrs<float> &Fin, const FieldPtrs<float> &Fout, const GridArgs<float> &G, void *s)
{
    if (G.ade_n <= 0) return;
    k_ade_post<<<(G.ade_n + 127) / 128, 128, 0, (cudaStream_t)s>>>(Fin, Fout, G);
}

void launch_post_fused(const FieldPtrs<float> &Fin, const FieldPtrs<float> &Fout, const GridArgs<float> &G,
                       const PostArgs &Q, void *s)
{
    const int nb = Q.nb_ade + Q.nb_plane + Q.nb_inj;
    if (nb <= 0) return;
    k_post_fused<<<nb, 128, 0, (cudaStream_t)s>>>(Fin, Fout, G, Q);
}

}  // namespace omx
