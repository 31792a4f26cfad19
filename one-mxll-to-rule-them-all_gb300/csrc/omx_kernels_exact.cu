// omx_kernels_exact.cu -- FP64 plain path (reference arithmetic) and the FP64 sparse kernels
// used by both paths.  Compiled with -fmad=false: no multiply-add contraction, so every
// expression rounds exactly as the FP64 CPU restatement does.
#include <cuda_runtime.h>
#include "omx_stencil.cuh"
#include "omx_sparse.cuh"
#include "omx_batch.cuh"

namespace omx {

template <> void launch_h<double>(const FieldPtrs<double> &F, const GridArgs<double> &G, void *s)
{
    launch_h_impl<double, true>(F, G, s);
}
template <> void launch_e<double>(const FieldPtrs<double> &F, const GridArgs<double> &G, void *s)
{
    launch_e_impl<double, true>(F, G, s);
}

template <> void launch_batch3<double>(int pass, const BatchGrid<double> *g, int n, long long total, int kch,
                                      int blocks, void *s)
{
    launch_batch3_impl<double, true>(pass, g, n, total, kch, blocks, s);
}
template <> int batch3_blocks<double>() { return batch3_blocks_impl<double, true>(); }
template <> void launch_ade<double>(const FieldPtrs<double> &F, const GridArgs<double> &G, void *s)
{
    if (G.ade_n > 0) k_ade<double><<<(G.ade_n + 127) / 128, 128, 0, (cudaStream_t)s>>>(F, G);
}
template <class R> void launch_src_batch(const BatchSrc<R> *e, int n, long long total, void *s)
{
    if (n <= 0 || total <= 0) return;
    k_src_batch<R><<<(unsigned)((total + 127) / 128), 128, 0, (cudaStream_t)s>>>(e, n, total);
}
template <class R> void launch_sample_batch(const BatchDet<R> *e, int n, long long total, void *s)
{
    if (n <= 0 || total <= 0) return;
    k_sample_batch<R><<<(unsigned)((total + 127) / 128), 128, 0, (cudaStream_t)s>>>(e, n, total);
}

template <class R> void launch_src(const FieldPtrs<R> &F, const SrcArgs &S, StepParam amp, void *s)
{
    if (S.n <= 0) return;
    k_src<R><<<(S.n + 127) / 128, 128, 0, (cudaStream_t)s>>>(F, S, amp);
}
template <class R> void launch_plane(const FieldPtrs<R> &F, const Lay &L, const PlaneArgs &P, StepParam amp, void *s)
{
    int n[3] = {L.nx, L.ny, L.nz};
    int ax0 = (P.axis == 0) ? 1 : 0;
    int ax1 = (P.axis == 2) ? 1 : 2;
    int nb = (L.dims == 2) ? 1 : n[ax1];
    dim3 g((n[ax0] + 127) / 128, nb, 1);
    k_plane<R><<<g, 128, 0, (cudaStream_t)s>>>(F, L, P, amp);
}
template <class R> void launch_inject(const FieldPtrs<R> &F, const JState &J, const InjArgs &I, StepParam t,
                                      StepParam ts, double dt_eps0, void *s)
{
    if (I.n <= 0) return;
    k_inject<R><<<(I.n + 127) / 128, 128, 0, (cudaStream_t)s>>>(F, J, I, t, ts, dt_eps0);
}
template <class R> void launch_emit(const FieldPtrs<R> &F, const Lay &L, const EmitArgs &A, StepParam move, void *s)
{
    if (A.n <= 0) return;
    // one warp per block: the FP64 work of a few thousand emitters spreads over every SM
    k_emit<R><<<(A.n + 31) / 32, 32, 0, (cudaStream_t)s>>>(F, L, A, move);
}
void launch_scatter(const JState &J, const ScatArgs &S, StepParam move, void *s)
{
    if (S.np <= 0) return;
    k_scatter<<<(S.np + 63) / 64, 64, 0, (cudaStream_t)s>>>(J, S, move);
}
template <class R> void launch_sample(const FieldPtrs<R> &F, const DetArgs &D, StepParam slot, StepParam time, void *s)
{
    const int n = D.n > 0 ? D.n : 1;
    k_sample<R><<<(n + 127) / 128, 128, 0, (cudaStream_t)s>>>(F, D, slot, time);
}
void launch_step_advance(int *step, void *s)
{
    k_step_advance<<<1, 32, 0, (cudaStream_t)s>>>(step);
}
void launch_cl_trajectories(const ClTrajArgs &A, void *s)
{
    if (A.n <= 0) return;
    k_cl_trajectories<<<(A.n + 63) / 64, 64, 0, (cudaStream_t)s>>>(A);
}
template <class R>
void launch_cl_gather(const FieldPtrs<R> &F, const Lay &L, const EmitArgs &A, const ClDeploy &D, StepParam move, void *s)
{
    k_cl_gather<R><<<(A.n + 127) / 128, 128, 0, (cudaStream_t)s>>>(F, L, A, D, move);
}
template void launch_cl_gather<float>(const FieldPtrs<float> &, const Lay &, const EmitArgs &, const ClDeploy &,
                                      StepParam, void *);
template void launch_cl_gather<double>(const FieldPtrs<double> &, const Lay &, const EmitArgs &, const ClDeploy &,
                                       StepParam, void *);
void launch_cl_subset_check_reseed(const EmitArgs &A, const ClDeploy &D, void *s)
{
    if (D.n_sub > 0) k_cl_subset<<<(D.n_sub + 31) / 32, 32, 0, (cudaStream_t)s>>>(A, D);
    k_cl_check<<<1, 1, 0, (cudaStream_t)s>>>(D);
    k_cl_reseed<<<(A.n + 31) / 32, 32, 0, (cudaStream_t)s>>>(A, D);
}
template <class R>
void launch_field_energy(const FieldPtrs<R> &F, const Lay &L, const int *used, double eps0, double mu0, double dV,
                         double *out, void *s)
{
    // out[0..303] holds the per-block partials (zeroed here), out[304] the sum
    constexpr int NB = 304;
    cudaMemsetAsync(out, 0, sizeof(double) * NB, (cudaStream_t)s);
    for (int c = 0; c < 6; ++c)
        if (used[c]) k_field_energy<R><<<NB, 256, 0, (cudaStream_t)s>>>(F, L, c, 0.5 * dV * (c < 3 ? eps0 : mu0), out);
    k_sum_parts<<<1, 32, 0, (cudaStream_t)s>>>(out, NB, out + NB);
}
template void launch_field_energy<float>(const FieldPtrs<float> &, const Lay &, const int *, double, double, double,
                                         double *, void *);
template void launch_field_energy<double>(const FieldPtrs<double> &, const Lay &, const int *, double, double, double,
                                          double *, void *);
void launch_flush(float *buf, long long n, void *s)
{
    k_flush<<<152 * 8, 256, 0, (cudaStream_t)s>>>(buf, n);
}

#define OMX_INST(R)                                                                                      \
    template void launch_src<R>(const FieldPtrs<R> &, const SrcArgs &, StepParam, void *);                \
    template void launch_plane<R>(const FieldPtrs<R> &, const Lay &, const PlaneArgs &, StepParam, void *); \
    template void launch_inject<R>(const FieldPtrs<R> &, const JState &, const InjArgs &, StepParam,      \
                                   StepParam, double, void *);                                           \
    template void launch_emit<R>(const FieldPtrs<R> &, const Lay &, const EmitArgs &, StepParam, void *); \
    template void launch_sample<R>(const FieldPtrs<R> &, const DetArgs &, StepParam, StepParam, void *); \
    template void launch_src_batch<R>(const BatchSrc<R> *, int, long long, void *);                      \
    template void launch_sample_batch<R>(const BatchDet<R> *, int, long long, void *);
OMX_INST(float)
OMX_INST(double)

}  // namespace omx
