// omx_stencil.cuh -- Yee H/E updates with the CPML psi recursion and the Drude / Drude-Lorentz
// auxiliary differential equations fused into one pass per half-step (1D, 2D TMz/TEz, 3D).
//
// Each routine restates the reference's loop body (paths relative to the reference root):
//   3D  src/FDTD/mxll_3D_mod.f90:505-923   2D  src/FDTD/mxll_2D_mod.f90:450-864
//   1D  src/FDTD/mxll_1D_mod.f90:252-355   ADE src/FDTD/classical_medium_mod.f90:773-833
// The reference updates the bulk first and then adds the CPML corrections face by face
// (x-lo, x-hi, y-lo, y-hi, z-lo, z-hi).  psi depends only on the other field, which is not
// written in the same half-step, so a single pass that adds the corrections of one cell in
// that face order produces the same values.  With EXACT (FP64 path, compiled without FMA
// contraction) every expression keeps the reference's operand order; the FP32 path folds
// 1/dr into the CPML c coefficients and lets the compiler contract multiply-adds.
//
// Thread mapping: 32 consecutive i per warp (coalesced rows), each thread marches along the
// slowest axis (k in 3D, j in 2D) over a chunk of KCH cells and carries the neighbour value it
// already loaded into the next iteration, so each field value is read from memory once.
#pragma once
#include "omx_internal.h"
#include "omx_post.cuh"

namespace omx {

template <class R, bool EXACT>
__device__ __forceinline__ R psi3(R b, R psi, R c, R d, R dr)
{
    if (EXACT) return b * psi + c * d / dr;     // bh*psi + ch*(E(i+1)-E(i))/dr
    return b * psi + c * d;
}
template <class R, bool EXACT>
__device__ __forceinline__ R psi2(R b, R psi, R c, R d, R dr)
{
    if (EXACT) return b * psi + c * (d / dr);   // rot = (E(i+1)-E(i))/dr ; bh*psi + ch*rot
    return b * psi + c * d;
}

// Auxiliary-differential-equation update of one dispersive E component
// (get_medium_polarization, classical_medium_mod.f90:773-833).  ADE state lives at
// ade[(c*(2+2P) + slot)*bbV + b].
template <class R>
__device__ __forceinline__ R ade_update(R e, R rot, const ClsR<R> &cl, int c, long long b, const GridArgs<R> &G)
{
    const MedR<R> &m = G.med[cl.medium];
    R *st = G.ade + (long long)c * (2 + 2 * G.P) * G.bbV + b;
    const R PD = st[0];
    if (cl.type == CLS_DRUDE) {
        const R t = m.C1 * e + m.C3 * rot - m.C4 * PD;
        st[0] = m.A1 * PD + m.A2 * (t + e);
        return t;
    }
    const long long V = G.bbV;
    const R eo = st[V];
    R t = m.C1 * e + m.C2 * eo + m.C3 * rot - m.C4 * PD;
    R pl[8], plo[8];
#pragma unroll
    for (int p = 0; p < 8; ++p) {
        if (p < m.np) {
            pl[p] = st[(2 + p) * V];
            plo[p] = st[(2 + G.P + p) * V];
            t = t - m.B1[p] * pl[p] - m.B2[p] * plo[p];
        }
    }
    st[0] = m.A1 * PD + m.A2 * (t + e);
#pragma unroll
    for (int p = 0; p < 8; ++p) {
        if (p < m.np) {
            const R nw = m.al[p] * pl[p] + m.be[p] * plo[p] + m.ga[p] * (t - eo);
            st[(2 + G.P + p) * V] = pl[p];
            st[(2 + p) * V] = nw;
        }
    }
    st[V] = e;
    return t;
}

// Bulk update of one E component inside the media box.  Vacuum and dielectric classes update
// here (E + dt_eps0*eps_inv*rotH); dispersive classes were already advanced by k_ade in this
// half-step and only receive their CPML terms from the bulk pass.
template <class R>
__device__ __forceinline__ R plain_update(R e, R rot, int cls_id, const GridArgs<R> &G)
{
    const ClsR<R> cl = G.cls[cls_id];
    return cl.type == CLS_PLAIN ? e + cl.coef * rot : e;
}

// curl H of component c at (i,j,k) with the bulk kernels' expressions and periodic remaps
template <class R>
__device__ __forceinline__ R curl_h(const FieldPtrs<R> &F, const GridArgs<R> &G, int c, int i, int j, int k)
{
    const Lay &L = G.L;
    const long long idx = L.off + i + (long long)L.px * j + L.pz * k;
    const long long mx = (i == 1 && G.per[0]) ? (long long)(L.nx - 1) : -1LL;
    if (L.dims == 1) return (F.f[4][idx - 1] - F.f[4][idx]) * G.den_e[0][i];
    const long long my = (j == 1 && G.per[1]) ? (long long)(L.ny - 1) * L.px : -(long long)L.px;
    if (L.dims == 2) {
        if (G.mode2d == 1)
            return (F.f[4][idx] - F.f[4][idx + mx]) * G.den_e[0][i] + (F.f[3][idx + my] - F.f[3][idx]) * G.den_e[1][j];
        if (c == 0) return (F.f[5][idx] - F.f[5][idx + my]) * G.den_e[1][j];
        return (F.f[5][idx + mx] - F.f[5][idx]) * G.den_e[0][i];
    }
    const long long mz = (k == 1 && G.per[2]) ? (long long)(L.nz - 1) * L.pz : -L.pz;
    if (c == 0)
        return (F.f[5][idx] - F.f[5][idx + my]) * G.den_e[1][j] + (F.f[4][idx + mz] - F.f[4][idx]) * G.den_e[2][k];
    if (c == 1)
        return (F.f[5][idx + mx] - F.f[5][idx]) * G.den_e[0][i] + (F.f[3][idx] - F.f[3][idx + mz]) * G.den_e[2][k];
    return (F.f[4][idx] - F.f[4][idx + mx]) * G.den_e[0][i] + (F.f[3][idx + my] - F.f[3][idx]) * G.den_e[1][j];
}

// Dispersive cells (compact list): the ADE part of the E update, run before the bulk pass.
template <class R>
__global__ void k_ade(FieldPtrs<R> F, GridArgs<R> G)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= G.ade_n) return;
    const int4 en = G.ade_ent[q];
    const int b = G.ade_b[q];
    const int c = en.w;
    const R rot = curl_h<R>(F, G, c, en.x, en.y, en.z);
    const Lay &L = G.L;
    const long long idx = L.off + en.x + (long long)L.px * en.y + L.pz * en.z;
    const ClsR<R> cl = G.cls[G.mat[c][b]];
    R *E = F.f[c];
    E[idx] = ade_update<R>(E[idx], rot, cl, c, b, G);
}

// ===================================================================================== 3D
// One 32 x 4 x kch tile of the pass at block coordinates (bx, by, bz): the single-grid
// kernel passes its block index, the batched kernel a tile of its work list.
template <class R, bool EXACT>
__device__ __forceinline__ void h3_tile(const FieldPtrs<R> &F, const GridArgs<R> &G, int kch, int bx, int by, int bz)
{
    const Lay L = G.L;
    const int i = 1 + bx * blockDim.x + threadIdx.x;
    const int j = 1 + by * blockDim.y + threadIdx.y;
    if (G.step_inc && i == 1 && j == 1 && bz == 0) *G.step_inc += 1;   // device-loop step counter
    if (i > L.nx || j > L.ny) return;
    const int k0 = 1 + bz * kch;
    const int k1 = min(L.nz, k0 + kch - 1);
    R *__restrict__ Ex = F.f[0];
    R *__restrict__ Ey = F.f[1];
    R *__restrict__ Ez = F.f[2];
    R *__restrict__ Hx = F.f[3];
    R *__restrict__ Hy = F.f[4];
    R *__restrict__ Hz = F.f[5];
    const long long sx = (i == L.nx && G.per[0]) ? (long long)(1 - L.nx) : 1LL;
    const long long sy = (j == L.ny && G.per[1]) ? (long long)(1 - L.ny) * L.px : (long long)L.px;
    const R dhx = G.den_h[0][i], dhy = G.den_h[1][j];
    const int lx = G.lH[0][i], ly = G.lH[1][j];
    const R dt_mu0 = G.dt_mu0, dr = G.dr;
    long long idx = L.off + i + (long long)L.px * j + L.pz * k0;
    R ex_c = Ex[idx], ey_c = Ey[idx];
#pragma unroll 2   // two planes of loads in flight (the E pass is faster without)
    for (int k = k0; k <= k1; ++k, idx += L.pz) {
        const long long sz = (k == L.nz && G.per[2]) ? (long long)(1 - L.nz) * L.pz : L.pz;
        const R ez_c = Ez[idx], ez_jp = Ez[idx + sy], ez_ip = Ez[idx + sx];
        const R ey_kp = Ey[idx + sz], ey_ip = Ey[idx + sx];
        const R ex_kp = Ex[idx + sz], ex_jp = Ex[idx + sy];
        const R dhz = G.den_h[2][k];
        // the old H of this cell is read by this thread only: streaming loads and stores
        R hx = __ldcs(Hx + idx) + dt_mu0 * ((ez_c - ez_jp) * dhy + (ey_kp - ey_c) * dhz);
        R hy = __ldcs(Hy + idx) + dt_mu0 * ((ez_ip - ez_c) * dhx + (ex_c - ex_kp) * dhz);
        R hz = __ldcs(Hz + idx) + dt_mu0 * ((ey_c - ey_ip) * dhx + (ex_jp - ex_c) * dhy);
        if (lx >= 0) {  // mxll_3D_mod.f90:585-620
            const long long p = lx + (long long)G.L2 * ((j - 1) + (long long)L.ny * (k - 1));
            const R b = G.bH[0][i], c = G.cH[0][i];
            const R v0 = psi3<R, EXACT>(b, G.psiH[0][0][p], c, ez_ip - ez_c, dr);
            const R v1 = psi3<R, EXACT>(b, G.psiH[0][1][p], c, ey_c - ey_ip, dr);
            G.psiH[0][0][p] = v0;
            G.psiH[0][1][p] = v1;
            hy = hy + dt_mu0 * v0;
            hz = hz + dt_mu0 * v1;
        }
        if (ly >= 0) {  // :622-657
            const long long p = (i - 1) + (long long)L.nx * (ly + (long long)G.L2 * (k - 1));
            const R b = G.bH[1][j], c = G.cH[1][j];
            const R v0 = psi3<R, EXACT>(b, G.psiH[1][0][p], c, ez_c - ez_jp, dr);
            const R v1 = psi3<R, EXACT>(b, G.psiH[1][1][p], c, ex_jp - ex_c, dr);
            G.psiH[1][0][p] = v0;
            G.psiH[1][1][p] = v1;
            hx = hx + dt_mu0 * v0;
            hz = hz + dt_mu0 * v1;
        }
        const int lz = G.lH[2][k];
        if (lz >= 0) {  // :659-694
            const long long p = (i - 1) + (long long)L.nx * ((j - 1) + (long long)L.ny * lz);
            const R b = G.bH[2][k], c = G.cH[2][k];
            const R v0 = psi3<R, EXACT>(b, G.psiH[2][0][p], c, ey_kp - ey_c, dr);
            const R v1 = psi3<R, EXACT>(b, G.psiH[2][1][p], c, ex_c - ex_kp, dr);
            G.psiH[2][0][p] = v0;
            G.psiH[2][1][p] = v1;
            hx = hx + dt_mu0 * v0;
            hy = hy + dt_mu0 * v1;
        }
        __stcs(Hx + idx, hx);
        __stcs(Hy + idx, hy);
        __stcs(Hz + idx, hz);
        // periodic ghost planes H(0) = H(n) (mxll_3D_mod.f90:725-738); the wraps run one after the
        // other over whole planes, so a corner ghost ends up equal to H(n, n, .) as well
        const bool gx = G.per[0] && i == L.nx, gy = G.per[1] && j == L.ny, gz = G.per[2] && k == L.nz;
        if (gx | gy | gz) {
            const long long ox = gx ? -(long long)L.nx : 0, oy = gy ? -(long long)L.ny * L.px : 0;
            const long long oz = gz ? -(long long)L.nz * L.pz : 0;
            if (gy) Hx[idx + oy] = hx;
            if (gz) Hx[idx + oz] = hx;
            if (gy && gz) Hx[idx + oy + oz] = hx;
            if (gx) Hy[idx + ox] = hy;
            if (gz) Hy[idx + oz] = hy;
            if (gx && gz) Hy[idx + ox + oz] = hy;
            if (gx) Hz[idx + ox] = hz;
            if (gy) Hz[idx + oy] = hz;
            if (gx && gy) Hz[idx + ox + oy] = hz;
        }
        ex_c = ex_kp;
        ey_c = ey_kp;
    }
}

// FP32: at most 48 registers, 10 blocks per SM (measured 8 % faster than the unbounded 64
// registers at 512^3; the E pass takes its own bound, 9 blocks)
template <class R, bool EXACT>
__global__ void __launch_bounds__(128, (sizeof(R) == 4 ? 10 : 1)) k_h3(FieldPtrs<R> F, GridArgs<R> G, int kch)
{
    h3_tile<R, EXACT>(F, G, kch, blockIdx.x, blockIdx.y, blockIdx.z);
}

// One 32 x 4 x kch tile of the pass at block coordinates (bx, by, bz): the single-grid
// kernel passes its block index, the batched kernel a tile of its work list.
template <class R, bool EXACT>
__device__ __forceinline__ void e3_tile(const FieldPtrs<R> &F, const GridArgs<R> &G, int kch, int bx, int by, int bz)
{
    const Lay L = G.L;
    const int i = 1 + bx * blockDim.x + threadIdx.x;
    const int j = 1 + by * blockDim.y + threadIdx.y;
    if (i > L.nx || j > L.ny) return;
    const int k0 = 1 + bz * kch;
    const int k1 = min(L.nz, k0 + kch - 1);
    R *__restrict__ Ex = F.f[0];
    R *__restrict__ Ey = F.f[1];
    R *__restrict__ Ez = F.f[2];
    R *__restrict__ Hx = F.f[3];
    R *__restrict__ Hy = F.f[4];
    R *__restrict__ Hz = F.f[5];
    const long long mx = (i == 1 && G.per[0]) ? (long long)(L.nx - 1) : -1LL;
    const long long my = (j == 1 && G.per[1]) ? (long long)(L.ny - 1) * L.px : -(long long)L.px;
    const R dex = G.den_e[0][i], dey = G.den_e[1][j];
    const int lx = G.lE[0][i], ly = G.lE[1][j];
    const R dt_eps0 = G.dt_eps0, dr = G.dr;
    const bool bb_ij = (i >= G.bb0[0] && i <= G.bb1[0] && j >= G.bb0[1] && j <= G.bb1[1]);
    long long idx = L.off + i + (long long)L.px * j + L.pz * k0;
    const long long mz0 = (k0 == 1 && G.per[2]) ? (long long)(L.nz - 1) * L.pz : -L.pz;
    R hx_km = Hx[idx + mz0], hy_km = Hy[idx + mz0];
    for (int k = k0; k <= k1; ++k, idx += L.pz) {
        const R hx_c = Hx[idx], hy_c = Hy[idx], hz_c = Hz[idx];
        const R hz_jm = Hz[idx + my], hz_im = Hz[idx + mx];
        const R hy_im = Hy[idx + mx], hx_jm = Hx[idx + my];
        const R dez = G.den_e[2][k];
        const R rx = (hz_c - hz_jm) * dey + (hy_km - hy_c) * dez;
        const R ry = (hz_im - hz_c) * dex + (hx_c - hx_km) * dez;
        const R rz = (hy_c - hy_im) * dex + (hx_jm - hx_c) * dey;
        R ex = __ldcs(Ex + idx), ey = __ldcs(Ey + idx), ez = __ldcs(Ez + idx);   // read by this thread only
        if (G.pl_on && (G.pl_axis == 0 ? i : (G.pl_axis == 1 ? j : k)) == G.pl_index) {
            // the plane source of this step (source_interactions before the E update)
            const double a = sp_get(G.pl_amp);
            if (a != 0.0) {
                const double add = __dmul_rn(G.pl_c_src, a);
                if (G.pl_comp == 0) ex = (R)__dadd_rn((double)ex, add);
                else if (G.pl_comp == 1) ey = (R)__dadd_rn((double)ey, add);
                else ez = (R)__dadd_rn((double)ez, add);
            }
        }
        if (bb_ij && k >= G.bb0[2] && k <= G.bb1[2]) {
            const long long b = (i - G.bb0[0]) + (long long)G.bbd[0] * ((j - G.bb0[1]) + (long long)G.bbd[1] * (k - G.bb0[2]));
            ex = plain_update<R>(ex, rx, G.mat[0][b], G);
            ey = plain_update<R>(ey, ry, G.mat[1][b], G);
            ez = plain_update<R>(ez, rz, G.mat[2][b], G);
        } else {
            ex = ex + dt_eps0 * rx;
            ey = ey + dt_eps0 * ry;
            ez = ez + dt_eps0 * rz;
        }
        if (lx >= 0) {  // mxll_3D_mod.f90:817-849
            const long long p = lx + (long long)G.L2 * ((j - 1) + (long long)L.ny * (k - 1));
            const R b = G.bE[0][i], c = G.cE[0][i];
            const R v0 = psi3<R, EXACT>(b, G.psiE[0][0][p], c, hz_im - hz_c, dr);
            const R v1 = psi3<R, EXACT>(b, G.psiE[0][1][p], c, hy_c - hy_im, dr);
            G.psiE[0][0][p] = v0;
            G.psiE[0][1][p] = v1;
            ey = ey + dt_eps0 * v0;
            ez = ez + dt_eps0 * v1;
        }
        if (ly >= 0) {  // :851-885
            const long long p = (i - 1) + (long long)L.nx * (ly + (long long)G.L2 * (k - 1));
            const R b = G.bE[1][j], c = G.cE[1][j];
            const R v0 = psi3<R, EXACT>(b, G.psiE[1][0][p], c, hz_c - hz_jm, dr);
            const R v1 = psi3<R, EXACT>(b, G.psiE[1][1][p], c, hx_jm - hx_c, dr);
            G.psiE[1][0][p] = v0;
            G.psiE[1][1][p] = v1;
            ex = ex + dt_eps0 * v0;
            ez = ez + dt_eps0 * v1;
        }
        const int lz = G.lE[2][k];
        if (lz >= 0) {  // :887-921
            const long long p = (i - 1) + (long long)L.nx * ((j - 1) + (long long)L.ny * lz);
            const R b = G.bE[2][k], c = G.cE[2][k];
            const R v0 = psi3<R, EXACT>(b, G.psiE[2][0][p], c, hy_km - hy_c, dr);
            const R v1 = psi3<R, EXACT>(b, G.psiE[2][1][p], c, hx_c - hx_km, dr);
            G.psiE[2][0][p] = v0;
            G.psiE[2][1][p] = v1;
            ex = ex + dt_eps0 * v0;
            ey = ey + dt_eps0 * v1;
        }
        __stcs(Ex + idx, ex);
        __stcs(Ey + idx, ey);
        __stcs(Ez + idx, ez);
        hx_km = hx_c;
        hy_km = hy_c;
    }
}

// FP32: at most 56 registers, 9 blocks per SM (4 % faster than the unbounded 64 registers at
// 512^3 and 256^3)
template <class R, bool EXACT>
__global__ void __launch_bounds__(128, (sizeof(R) == 4 ? 9 : 1)) k_e3(FieldPtrs<R> F, GridArgs<R> G, int kch)
{
    e3_tile<R, EXACT>(F, G, kch, blockIdx.x, blockIdx.y, blockIdx.z);
}

// ===================================================================================== 2D
// TMz (Ez, Hx, Hy): mxll_2D_mod.f90:469-554 and :661-750.
// TEz (Ex, Ey, Hz): :556-634 and :752-862.
template <class R, bool EXACT>
__global__ void __launch_bounds__(128) k_h2(FieldPtrs<R> F, GridArgs<R> G, int jch)
{
    const Lay L = G.L;
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (G.step_inc && i == 1 && blockIdx.y == 0) *G.step_inc += 1;   // device-loop step counter
    if (i > L.nx) return;
    const int j0 = 1 + blockIdx.y * jch;
    const int j1 = min(L.ny, j0 + jch - 1);
    const long long sx = (i == L.nx && G.per[0]) ? (long long)(1 - L.nx) : 1LL;
    const R dhx = G.den_h[0][i];
    const int lx = G.lH[0][i];
    const R dt_mu0 = G.dt_mu0, dr = G.dr;
    long long idx = L.off + i + (long long)L.px * j0;
    if (G.mode2d == 1) {
        R *__restrict__ Ez = F.f[2];
        R *__restrict__ Hx = F.f[3];
        R *__restrict__ Hy = F.f[4];
        R ez_c = Ez[idx];
        for (int j = j0; j <= j1; ++j, idx += L.px) {
            const long long sy = (j == L.ny && G.per[1]) ? (long long)(1 - L.ny) * L.px : (long long)L.px;
            const R ez_jp = Ez[idx + sy], ez_ip = Ez[idx + sx];
            R hx = Hx[idx] + dt_mu0 * ((ez_c - ez_jp) * G.den_h[1][j]);
            R hy = Hy[idx] + dt_mu0 * ((ez_ip - ez_c) * dhx);
            if (lx >= 0) {
                const long long p = lx + (long long)G.L2 * (j - 1);
                const R v = psi2<R, EXACT>(G.bH[0][i], G.psiH[0][0][p], G.cH[0][i], ez_ip - ez_c, dr);
                G.psiH[0][0][p] = v;
                hy = hy + dt_mu0 * v;
            }
            const int ly = G.lH[1][j];
            if (ly >= 0) {
                const long long p = (i - 1) + (long long)L.nx * ly;
                const R v = psi2<R, EXACT>(G.bH[1][j], G.psiH[1][0][p], G.cH[1][j], ez_c - ez_jp, dr);
                G.psiH[1][0][p] = v;
                hx = hx + dt_mu0 * v;
            }
            Hx[idx] = hx;
            Hy[idx] = hy;
            // periodic ghosts Hy(0,:) = Hy(nx,:), Hx(:,0) = Hx(:,ny) (mxll_2D_mod.f90:666-672)
            if (G.per[0] && i == L.nx) Hy[idx - L.nx] = hy;
            if (G.per[1] && j == L.ny) Hx[idx - (long long)L.ny * L.px] = hx;
            ez_c = ez_jp;
        }
    } else {
        R *__restrict__ Ex = F.f[0];
        R *__restrict__ Ey = F.f[1];
        R *__restrict__ Hz = F.f[5];
        R ex_c = Ex[idx];
        for (int j = j0; j <= j1; ++j, idx += L.px) {
            const long long sy = (j == L.ny && G.per[1]) ? (long long)(1 - L.ny) * L.px : (long long)L.px;
            const R ey_c = Ey[idx], ey_ip = Ey[idx + sx], ex_jp = Ex[idx + sy];
            R hz = Hz[idx] + dt_mu0 * ((ey_c - ey_ip) * dhx + (ex_jp - ex_c) * G.den_h[1][j]);
            if (lx >= 0) {
                const long long p = lx + (long long)G.L2 * (j - 1);
                const R v = psi2<R, EXACT>(G.bH[0][i], G.psiH[0][0][p], G.cH[0][i], ey_c - ey_ip, dr);
                G.psiH[0][0][p] = v;
                hz = hz + dt_mu0 * v;
            }
            const int ly = G.lH[1][j];
            if (ly >= 0) {
                const long long p = (i - 1) + (long long)L.nx * ly;
                const R v = psi2<R, EXACT>(G.bH[1][j], G.psiH[1][0][p], G.cH[1][j], ex_jp - ex_c, dr);
                G.psiH[1][0][p] = v;
                hz = hz + dt_mu0 * v;
            }
            Hz[idx] = hz;
            // periodic ghosts Hz(0,:) = Hz(nx,:) then Hz(:,0) = Hz(:,ny) (mxll_2D_mod.f90:757-763)
            {
                const bool gx = G.per[0] && i == L.nx, gy = G.per[1] && j == L.ny;
                if (gx) Hz[idx - L.nx] = hz;
                if (gy) Hz[idx - (long long)L.ny * L.px] = hz;
                if (gx && gy) Hz[idx - L.nx - (long long)L.ny * L.px] = hz;
            }
            ex_c = ex_jp;
        }
    }
}

template <class R, bool EXACT>
__global__ void __launch_bounds__(128) k_e2(FieldPtrs<R> F, GridArgs<R> G, int jch)
{
    const Lay L = G.L;
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i > L.nx) return;
    const int j0 = 1 + blockIdx.y * jch;
    const int j1 = min(L.ny, j0 + jch - 1);
    const long long mx = (i == 1 && G.per[0]) ? (long long)(L.nx - 1) : -1LL;
    const R dex = G.den_e[0][i];
    const int lx = G.lE[0][i];
    const R dt_eps0 = G.dt_eps0, dr = G.dr;
    const bool bb_i = (i >= G.bb0[0] && i <= G.bb1[0]);
    long long idx = L.off + i + (long long)L.px * j0;
    const long long my0 = (j0 == 1 && G.per[1]) ? (long long)(L.ny - 1) * L.px : -(long long)L.px;
    if (G.mode2d == 1) {
        R *__restrict__ Ez = F.f[2];
        R *__restrict__ Hx = F.f[3];
        R *__restrict__ Hy = F.f[4];
        R hx_jm = Hx[idx + my0];
        for (int j = j0; j <= j1; ++j, idx += L.px) {
            const R hx_c = Hx[idx], hy_c = Hy[idx], hy_im = Hy[idx + mx];
            const R r = (hy_c - hy_im) * dex + (hx_jm - hx_c) * G.den_e[1][j];
            R ez = Ez[idx];
            if (bb_i && j >= G.bb0[1] && j <= G.bb1[1]) {
                const long long b = (i - G.bb0[0]) + (long long)G.bbd[0] * (j - G.bb0[1]);
                ez = plain_update<R>(ez, r, G.mat[2][b], G);
            } else {
                ez = ez + dt_eps0 * r;
            }
            if (lx >= 0) {
                const long long p = lx + (long long)G.L2 * (j - 1);
                const R v = psi2<R, EXACT>(G.bE[0][i], G.psiE[0][0][p], G.cE[0][i], hy_c - hy_im, dr);
                G.psiE[0][0][p] = v;
                ez = ez + dt_eps0 * v;
            }
            const int ly = G.lE[1][j];
            if (ly >= 0) {
                const long long p = (i - 1) + (long long)L.nx * ly;
                const R v = psi2<R, EXACT>(G.bE[1][j], G.psiE[1][0][p], G.cE[1][j], hx_jm - hx_c, dr);
                G.psiE[1][0][p] = v;
                ez = ez + dt_eps0 * v;
            }
            Ez[idx] = ez;
            hx_jm = hx_c;
        }
    } else {
        R *__restrict__ Ex = F.f[0];
        R *__restrict__ Ey = F.f[1];
        R *__restrict__ Hz = F.f[5];
        R hz_jm = Hz[idx + my0];
        for (int j = j0; j <= j1; ++j, idx += L.px) {
            const R hz_c = Hz[idx], hz_im = Hz[idx + mx];
            const R rx = (hz_c - hz_jm) * G.den_e[1][j];
            const R ry = (hz_im - hz_c) * dex;
            R ex = Ex[idx], ey = Ey[idx];
            if (bb_i && j >= G.bb0[1] && j <= G.bb1[1]) {
                const long long b = (i - G.bb0[0]) + (long long)G.bbd[0] * (j - G.bb0[1]);
                ex = plain_update<R>(ex, rx, G.mat[0][b], G);
                ey = plain_update<R>(ey, ry, G.mat[1][b], G);
            } else {
                ex = ex + dt_eps0 * rx;
                ey = ey + dt_eps0 * ry;
            }
            if (lx >= 0) {
                const long long p = lx + (long long)G.L2 * (j - 1);
                const R v = psi2<R, EXACT>(G.bE[0][i], G.psiE[0][0][p], G.cE[0][i], hz_im - hz_c, dr);
                G.psiE[0][0][p] = v;
                ey = ey + dt_eps0 * v;
            }
            const int ly = G.lE[1][j];
            if (ly >= 0) {
                const long long p = (i - 1) + (long long)L.nx * ly;
                const R v = psi2<R, EXACT>(G.bE[1][j], G.psiE[1][0][p], G.cE[1][j], hz_c - hz_jm, dr);
                G.psiE[1][0][p] = v;
                ex = ex + dt_eps0 * v;
            }
            Ex[idx] = ex;
            Ey[idx] = ey;
            hz_jm = hz_c;
        }
    }
}

// ===================================================================================== 1D
// Ex(1:n), Hy(1:n-1) on the single axis (mxll_1D_mod.f90:252-355).
template <class R, bool EXACT>
__global__ void k_h1(FieldPtrs<R> F, GridArgs<R> G)
{
    const Lay L = G.L;
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (G.step_inc && i == 1) *G.step_inc += 1;   // device-loop step counter
    if (i > L.nx - 1) return;
    R *__restrict__ Ex = F.f[0];
    R *__restrict__ Hy = F.f[4];
    const long long idx = L.off + i;
    const R d = Ex[idx] - Ex[idx + 1];
    R hy = Hy[idx] + G.dt_mu0 * d * G.den_h[0][i];
    const int l = G.lH[0][i];
    if (l >= 0) {
        const R v = psi3<R, EXACT>(G.bH[0][i], G.psiH[0][0][l], G.cH[0][i], d, G.dr);
        G.psiH[0][0][l] = v;
        hy = hy + G.dt_mu0 * v;
    }
    Hy[idx] = hy;
}

template <class R, bool EXACT>
__global__ void k_e1(FieldPtrs<R> F, GridArgs<R> G)
{
    const Lay L = G.L;
    const int i = 2 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i > L.nx - 1) return;
    R *__restrict__ Ex = F.f[0];
    R *__restrict__ Hy = F.f[4];
    const long long idx = L.off + i;
    const R d = Hy[idx - 1] - Hy[idx];
    const R r = d * G.den_e[0][i];
    R ex = Ex[idx];
    if (i >= G.bb0[0] && i <= G.bb1[0]) {
        const long long b = i - G.bb0[0];
        ex = plain_update<R>(ex, r, G.mat[0][b], G);
    } else {
        ex = ex + G.dt_eps0 * r;
    }
    const int l = G.lE[0][i];
    if (l >= 0) {
        const R v = psi2<R, EXACT>(G.bE[0][i], G.psiE[0][0][l], G.cE[0][i], d, G.dr);
        G.psiE[0][0][l] = v;
        ex = ex + G.dt_eps0 * v;
    }
    Ex[idx] = ex;
}

// ===================================================================================== launchers
constexpr int KCH3 = 16;   // planes marched per 3D thread
constexpr int JCH2 = 32;   // rows marched per 2D thread

template <class R, bool EXACT>
void launch_h_impl(const FieldPtrs<R> &F, const GridArgs<R> &G, void *stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    const Lay &L = G.L;
    if (L.dims == 3) {
        const int m = G.march > 0 ? G.march : KCH3;
        dim3 b(32, 4, 1), g((L.nx + 31) / 32, (L.ny + 3) / 4, (L.nz + m - 1) / m);
        k_h3<R, EXACT><<<g, b, 0, s>>>(F, G, m);
    } else if (L.dims == 2) {
        const int m = G.march > 0 ? G.march : JCH2;
        dim3 b(128, 1, 1), g((L.nx + 127) / 128, (L.ny + m - 1) / m, 1);
        k_h2<R, EXACT><<<g, b, 0, s>>>(F, G, m);
    } else {
        k_h1<R, EXACT><<<(L.nx + 127) / 128, 128, 0, s>>>(F, G);
    }
}

template <class R, bool EXACT>
void launch_e_impl(const FieldPtrs<R> &F, const GridArgs<R> &G, void *stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    const Lay &L = G.L;
    if (G.ade_n > 0) k_ade<R><<<(G.ade_n + 127) / 128, 128, 0, s>>>(F, G);
    if (L.dims == 3) {
        const int m = G.march > 0 ? G.march : KCH3;
        dim3 b(32, 4, 1), g((L.nx + 31) / 32, (L.ny + 3) / 4, (L.nz + m - 1) / m);
        k_e3<R, EXACT><<<g, b, 0, s>>>(F, G, m);
    } else if (L.dims == 2) {
        const int m = G.march > 0 ? G.march : JCH2;
        dim3 b(128, 1, 1), g((L.nx + 127) / 128, (L.ny + m - 1) / m, 1);
        k_e2<R, EXACT><<<g, b, 0, s>>>(F, G, m);
    } else {
        k_e1<R, EXACT><<<(L.nx + 127) / 128, 128, 0, s>>>(F, G);
    }
}

}  // namespace omx
