// omx_post.cuh -- per-cell source and current terms of the E update, shared by both kernel
// translation units and by several kernels (the separate source / current kernels, the merged
// launch after a fused pass, the 3D bulk E pass): the step-parameter read, the plane source and
// the emitter-current term.  They are written with explicit round-to-nearest operations, so a
// unit compiled with FMA contraction gives the same bits as the contraction-free unit (FP64
// arithmetic, as the reference's).
#pragma once
#include "omx_internal.h"

namespace omx {

__device__ __forceinline__ double sp_get(const StepParam &p)
{
    return p.tab ? p.tab[(long long)(*p.step) * p.stride] : p.val;
}

// Plane-wave soft source (extension): E_comp += c_src*amp at cell (a, b) of the plane, a along
// the first in-plane axis, b along the second (0 in 2D).
template <class R>
__device__ __forceinline__ void plane_point(const FieldPtrs<R> &F, const Lay &L, const PlaneArgs &P, double amp, int a,
                                            int b)
{
    const int n[3] = {L.nx, L.ny, L.nz};
    const int ax0 = (P.axis == 0) ? 1 : 0;
    const int ax1 = (L.dims == 2) ? -1 : ((P.axis == 2) ? 1 : 2);
    if (a >= n[ax0]) return;
    int c[3] = {0, 0, 0};
    c[P.axis] = P.index;
    c[ax0] = a + 1;
    if (ax1 >= 0) {
        if (b >= n[ax1]) return;
        c[ax1] = b + 1;
    }
    R *E = F.f[P.comp];
    const long long e = L.off + c[0] + (long long)L.px * c[1] + L.pz * c[2];
    E[e] = (R)__dadd_rn((double)E[e], __dmul_rn(P.c_src, amp));
}

// Emitter current in the E update (mxll_3D_mod.f90:756-761 and the 2D/1D analogues):
// E -= dt_eps0 * Jav, Jav = 0.5*(J_old(i) + tt*dJ(i) + J_old(i+1) + tt*dJ(i+1)), tt = time - t_skip.
template <class R>
__device__ __forceinline__ void inject_point(const FieldPtrs<R> &F, const JState &J, const InjArgs &I, double tt,
                                             double dt_eps0, int q)
{
    const int c = I.comp[q];
    const int a = I.sa[q], b = I.sb[q];
    const double ao = (a >= 0) ? J.Jo[c][a] : 0.0, ad = (a >= 0) ? J.dJ[c][a] : 0.0;
    double jav = __dadd_rn(ao, __dmul_rn(tt, ad));
    if (I.avg) {
        const double bo = (b >= 0) ? J.Jo[c][b] : 0.0, bd = (b >= 0) ? J.dJ[c][b] : 0.0;
        jav = __dmul_rn(0.5, __dadd_rn(__dadd_rn(jav, bo), __dmul_rn(tt, bd)));
    }
    R *E = F.f[c];
    const long long e = I.eidx[q];
    E[e] = (R)__dsub_rn((double)E[e], __dmul_rn(dt_eps0, jav));
}

}  // namespace omx
