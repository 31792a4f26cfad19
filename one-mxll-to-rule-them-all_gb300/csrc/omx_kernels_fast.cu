// omx_kernels_fast.cu -- FP32 fused path of the Yee/CPML/ADE half-step kernels.  FP32 field
// state with FP64-precomputed coefficients rounded once to FP32; multiply-adds contract to FMA.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include "omx_batch.cuh"
#include "omx_fused2d.cuh"
#include "omx_fused3t.cuh"

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

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime (no link to libcuda)
static PFN_cuTensorMapEncodeTiled_v12000 f3t_encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// One FP32 component over the whole padded array: dims {px, ny + 2, nz + 2}, base at element
// i = -3 of row (0, 0) (off - 3: 16-byte aligned because element i = 1 is 128-byte aligned; the
// last element, off - 3 + px (ny + 2)(nz + 2) - 1, lies inside the allocation).  Reads past a
// dimension return zero.
bool encode_f3t_maps(F3tMaps *M, const FieldPtrs<float> &in, const Lay &L, int ty)
{
    auto fn = f3t_encode_fn();
    // a row must hold cells -3 .. nx+1 (the boxes start 3 cells before a tile; E of cell nx+1)
    if (!fn || L.dims != 3 || L.off < 3 || L.px < L.nx + 5) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)L.px, (cuuint64_t)(L.ny + 2), (cuuint64_t)(L.nz + 2)};
    const cuuint64_t strides[2] = {(cuuint64_t)L.px * 4u, (cuuint64_t)L.pz * 4u};
    const cuuint32_t box[3] = {(cuuint32_t)F3T_BX, (cuuint32_t)(ty + 2), 1u};
    const cuuint32_t es[3] = {1u, 1u, 1u};
    for (int c = 0; c < 6; ++c) {
        if (!in.f[c]) return false;
        void *base = const_cast<float *>(in.f[c] + (L.off - 3));
        if (fn(&M->m[c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    }
    return true;
}

// the largest dynamic shared memory set so far for a fused 3D kernel on this device (the
// attribute grows with the ring depth a launch asks for)
template <class K> static cudaError_t f3t_smem_attr(K kernel, int *have, int bytes)
{
    int dev = 0;
    cudaGetDevice(&dev);
    int &h = have[dev < FZ_MAX_DEV ? dev : 0];
    if (h >= bytes) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) h = bytes;
    return e;
}

template <int TY, int MODE>
static cudaError_t launch_f3t(const F3tMaps &M, const Fused3Args &A, const GridArgs<float> &G, const int4 *items,
                              int n, int nd, int *err, cudaStream_t s)
{
    using S = F3tShape<TY>;
    static int have[FZ_MAX_DEV] = {};
    const int bytes = S::smem(nd);
    const cudaError_t e = f3t_smem_attr(k_fused3_tma<TY, MODE>, have, bytes);
    if (e != cudaSuccess) return e;
    if (n <= 0) return cudaSuccess;
    k_fused3_tma<TY, MODE><<<(unsigned)n, S::THREADS, bytes, s>>>(M, A, G, items, nd, err);
    return cudaGetLastError();
}

cudaError_t launch_fused3t_general(const Fused3Args &A, const GridArgs<float> &G, int form, const int4 *items, int n,
                                   bool e_half, void *sv)
{
    if (n <= 0) return cudaSuccess;
    const cudaStream_t s = (cudaStream_t)sv;
    const int ty = f3t_rows(form);
    const dim3 b(32, (unsigned)ty);
    if (ty == 16) {
        if (e_half) k_f3g_e<16><<<(unsigned)n, b, 0, s>>>(A, G, items);
        else k_f3g_h<16><<<(unsigned)n, b, 0, s>>>(A, G, items);
    } else {
        if (e_half) k_f3g_e<8><<<(unsigned)n, b, 0, s>>>(A, G, items);
        else k_f3g_h<8><<<(unsigned)n, b, 0, s>>>(A, G, items);
    }
    return cudaGetLastError();
}

int f3t_smem_bytes(int form)
{
    return f3t_rows(form) == 16 ? F3tShape<16>::smem(f3t_ring(form)) : F3tShape<8>::smem(f3t_ring(form));
}

cudaError_t launch_fused3t_lean(const F3tMaps &M, const Fused3Args &A, const GridArgs<float> &G, int form,
                                const int4 *items, int n, int *err, void *sv)
{
    const int nd = f3t_ring(form);
    const cudaStream_t s = (cudaStream_t)sv;
    if (f3t_rows(form) == 16) return launch_f3t<16, F3T_LEAN_ONLY>(M, A, G, items, n, nd, err, s);
    return launch_f3t<8, F3T_LEAN_ONLY>(M, A, G, items, n, nd, err, s);
}

template <int TY>
static cudaError_t launch_f3t_batch(const F3tBatchGrid *grids, int n, long long blocks, int nd, int *err,
                                    cudaStream_t s)
{
    using S = F3tShape<TY>;
    static int have[FZ_MAX_DEV] = {};
    const int bytes = S::smem(nd);
    const cudaError_t e = f3t_smem_attr(k_fused3_batch<TY>, have, bytes);
    if (e != cudaSuccess) return e;
    if (n <= 0 || blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    k_fused3_batch<TY><<<(unsigned)blocks, S::THREADS, bytes, s>>>(grids, n, nd, err);
    return cudaGetLastError();
}

cudaError_t launch_fused3t_batch_split(const F3tBatchGrid *grids, const int4 *gen, int ngen, const int4 *lean, int nlean,
                                       int form, int parts, int *err, void *sv)
{
    const cudaStream_t s = (cudaStream_t)sv;
    const int ty = f3t_rows(form), nd = f3t_ring(form);
    const dim3 b(32, (unsigned)ty);
    if (ngen > 0 && (parts & 1)) {
        if (ty == 16) k_f3g_h_batch<16><<<(unsigned)ngen, b, 0, s>>>(grids, gen);
        else k_f3g_h_batch<8><<<(unsigned)ngen, b, 0, s>>>(grids, gen);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (nlean > 0 && (parts & 2)) {
        static int have16[FZ_MAX_DEV] = {}, have8[FZ_MAX_DEV] = {};
        if (ty == 16) {
            const int bytes = F3tShape<16>::smem(nd);
            const cudaError_t e = f3t_smem_attr(k_fused3_batch_lean<16>, have16, bytes);
            if (e != cudaSuccess) return e;
            k_fused3_batch_lean<16><<<(unsigned)nlean, F3tShape<16>::THREADS, bytes, s>>>(grids, lean, nd, err);
        } else {
            const int bytes = F3tShape<8>::smem(nd);
            const cudaError_t e = f3t_smem_attr(k_fused3_batch_lean<8>, have8, bytes);
            if (e != cudaSuccess) return e;
            k_fused3_batch_lean<8><<<(unsigned)nlean, F3tShape<8>::THREADS, bytes, s>>>(grids, lean, nd, err);
        }
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (ngen > 0 && (parts & 4)) {
        if (ty == 16) k_f3g_e_batch<16><<<(unsigned)ngen, b, 0, s>>>(grids, gen);
        else k_f3g_e_batch<8><<<(unsigned)ngen, b, 0, s>>>(grids, gen);
    }
    return cudaGetLastError();
}

cudaError_t launch_fused3t_batch(const F3tBatchGrid *grids, int n, long long blocks, int form, int *err, void *s)
{
    const int nd = f3t_ring(form);
    if (f3t_rows(form) == 16) return launch_f3t_batch<16>(grids, n, blocks, nd, err, (cudaStream_t)s);
    return launch_f3t_batch<8>(grids, n, blocks, nd, err, (cudaStream_t)s);
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
