// omx_fused3d.cuh -- FP32 fused time step in 3D: the H update (mxll_3D_mod.f90:505-696) and the
// E update (:700-923) of one step in a single pass over HBM.
//
// Each cell's six field words are read once and written once per step (12 words instead of the
// 18 of two half-step passes).  As in the 2D TMz pass, the pass reads the "in" buffer set and
// writes the "out" set (ping-pong, H psi included), so that the new H a cell's E update needs at
// i-1, j-1 and k-1 can come from a neighbour thread or be recomputed from buffers nobody writes
// during the pass:
//   * i-1: the lower lane of the warp (shuffle); lane 0 recomputes it;
//   * j-1: the thread row below in the block (shared memory, double-buffered by plane parity,
//     one block barrier per plane); the block's first row recomputes it;
//   * k-1: the thread's own previous plane (registers); the first plane recomputes it.
// E psi and the ADE state are touched by their owner only.  Dispersive cells are finished by
// k_ade_post afterwards, sources and the emitter current by their own kernels (they commute with
// the bulk update up to FP32 rounding).  The host offers this path (omx_set_step_form) only when no
// dispersive cell lies in a CPML slab and no source point lies in a dispersive cell, for
// nx % 32 == 0 and ny % F3_BY == 0 (every thread owns a cell and reaches every barrier).
//
// Measured on GB300 at 512^3 it is slower than the two unfused passes (2.9 ms against 2.15 ms
// per step): the recomputes of the halo, whose loads come from L2, stall the warps that own
// them and, through the barrier, the whole block.  It is therefore off by default in 3D.
#pragma once
#include "omx_stencil.cuh"

namespace omx {

// New H component C (0 x, 1 y, 2 z) at (i, j, k) from the in buffers: the zero ghost at a
// non-periodic index 0, the periodic image otherwise.  Reads psi, writes nothing.
template <int C>
__device__ __forceinline__ float f3_hnew(const Fused3Args &A, const GridArgs<float> &G, int i, int j, int k)
{
    const Lay &L = G.L;
    if (i == 0) {
        if (!G.per[0]) return 0.f;
        i = L.nx;
    }
    if (j == 0) {
        if (!G.per[1]) return 0.f;
        j = L.ny;
    }
    if (k == 0) {
        if (!G.per[2]) return 0.f;
        k = L.nz;
    }
    const long long idx = L.off + i + (long long)L.px * j + L.pz * k;
    const long long sx = (i == L.nx && G.per[0]) ? (long long)(1 - L.nx) : 1LL;
    const long long sy = (j == L.ny && G.per[1]) ? (long long)(1 - L.ny) * L.px : (long long)L.px;
    const long long sz = (k == L.nz && G.per[2]) ? (long long)(1 - L.nz) * L.pz : L.pz;
    const float *Ex = A.in.f[0], *Ey = A.in.f[1], *Ez = A.in.f[2];
    const float dt_mu0 = G.dt_mu0, dr = G.dr;
    if (C == 0) {
        const float ez_c = Ez[idx], ez_jp = Ez[idx + sy], ey_c = Ey[idx], ey_kp = Ey[idx + sz];
        float h = A.in.f[3][idx] + dt_mu0 * ((ez_c - ez_jp) * G.den_h[1][j] + (ey_kp - ey_c) * G.den_h[2][k]);
        const int ly = G.lH[1][j], lz = G.lH[2][k];
        if (ly >= 0) {
            const long long p = (i - 1) + (long long)L.nx * (ly + (long long)G.L2 * (k - 1));
            h = h + dt_mu0 * psi3<float, false>(G.bH[1][j], G.psiH[1][0][p], G.cH[1][j], ez_c - ez_jp, dr);
        }
        if (lz >= 0) {
            const long long p = (i - 1) + (long long)L.nx * ((j - 1) + (long long)L.ny * lz);
            h = h + dt_mu0 * psi3<float, false>(G.bH[2][k], G.psiH[2][0][p], G.cH[2][k], ey_kp - ey_c, dr);
        }
        return h;
    } else if (C == 1) {
        const float ez_c = Ez[idx], ez_ip = Ez[idx + sx], ex_c = Ex[idx], ex_kp = Ex[idx + sz];
        float h = A.in.f[4][idx] + dt_mu0 * ((ez_ip - ez_c) * G.den_h[0][i] + (ex_c - ex_kp) * G.den_h[2][k]);
        const int lx = G.lH[0][i], lz = G.lH[2][k];
        if (lx >= 0) {
            const long long p = lx + (long long)G.L2 * ((j - 1) + (long long)L.ny * (k - 1));
            h = h + dt_mu0 * psi3<float, false>(G.bH[0][i], G.psiH[0][0][p], G.cH[0][i], ez_ip - ez_c, dr);
        }
        if (lz >= 0) {
            const long long p = (i - 1) + (long long)L.nx * ((j - 1) + (long long)L.ny * lz);
            h = h + dt_mu0 * psi3<float, false>(G.bH[2][k], G.psiH[2][1][p], G.cH[2][k], ex_c - ex_kp, dr);
        }
        return h;
    } else {
        const float ey_c = Ey[idx], ey_ip = Ey[idx + sx], ex_c = Ex[idx], ex_jp = Ex[idx + sy];
        float h = A.in.f[5][idx] + dt_mu0 * ((ey_c - ey_ip) * G.den_h[0][i] + (ex_jp - ex_c) * G.den_h[1][j]);
        const int lx = G.lH[0][i], ly = G.lH[1][j];
        if (lx >= 0) {
            const long long p = lx + (long long)G.L2 * ((j - 1) + (long long)L.ny * (k - 1));
            h = h + dt_mu0 * psi3<float, false>(G.bH[0][i], G.psiH[0][1][p], G.cH[0][i], ey_c - ey_ip, dr);
        }
        if (ly >= 0) {
            const long long p = (i - 1) + (long long)L.nx * (ly + (long long)G.L2 * (k - 1));
            h = h + dt_mu0 * psi3<float, false>(G.bH[1][j], G.psiH[1][1][p], G.cH[1][j], ex_jp - ex_c, dr);
        }
        return h;
    }
}

// One block: 32 x F3_BY columns (i, j), each thread marching kch planes along k.
__global__ void __launch_bounds__(32 * F3_BY) k_fused3(Fused3Args A, GridArgs<float> G, int kch)
{
    __shared__ float sh_hz[2][F3_BY][32], sh_hx[2][F3_BY][32];
    const Lay &L = G.L;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i = 1 + blockIdx.x * 32 + tx;
    const int j = 1 + blockIdx.y * F3_BY + ty;
    if (G.step_inc && i == 1 && j == 1 && blockIdx.z == 0) *G.step_inc += 1;   // device-loop step counter
    const int k0 = 1 + blockIdx.z * kch;
    const int k1 = min(L.nz, k0 + kch - 1);
    const float *__restrict__ Ex = A.in.f[0];
    const float *__restrict__ Ey = A.in.f[1];
    const float *__restrict__ Ez = A.in.f[2];
    const float *__restrict__ Hx = A.in.f[3];
    const float *__restrict__ Hy = A.in.f[4];
    const float *__restrict__ Hz = A.in.f[5];
    float *__restrict__ oEx = A.out.f[0];
    float *__restrict__ oEy = A.out.f[1];
    float *__restrict__ oEz = A.out.f[2];
    float *__restrict__ oHx = A.out.f[3];
    float *__restrict__ oHy = A.out.f[4];
    float *__restrict__ oHz = A.out.f[5];
    const long long sx = (i == L.nx && G.per[0]) ? (long long)(1 - L.nx) : 1LL;
    const long long sy = (j == L.ny && G.per[1]) ? (long long)(1 - L.ny) * L.px : (long long)L.px;
    const float dhx = G.den_h[0][i], dhy = G.den_h[1][j], dex = G.den_e[0][i], dey = G.den_e[1][j];
    const int lhx = G.lH[0][i], lhy = G.lH[1][j], lex = G.lE[0][i], ley = G.lE[1][j];
    const float dt_mu0 = G.dt_mu0, dt_eps0 = G.dt_eps0, dr = G.dr;
    const bool bb_ij = (i >= G.bb0[0] && i <= G.bb1[0] && j >= G.bb0[1] && j <= G.bb1[1]);
    long long idx = L.off + i + (long long)L.px * j + L.pz * k0;
    float ex_c = Ex[idx], ey_c = Ey[idx];
    // new H of the plane below the first one
    float hx_km = f3_hnew<0>(A, G, i, j, k0 - 1), hy_km = f3_hnew<1>(A, G, i, j, k0 - 1);
    for (int k = k0; k <= k1; ++k, idx += L.pz) {
        // ---- H_new(i, j, k): the expressions of h3_tile, H psi into the out set
        const long long sz = (k == L.nz && G.per[2]) ? (long long)(1 - L.nz) * L.pz : L.pz;
        const float ez_c = Ez[idx], ez_jp = Ez[idx + sy], ez_ip = Ez[idx + sx];
        const float ey_kp = Ey[idx + sz], ey_ip = Ey[idx + sx];
        const float ex_kp = Ex[idx + sz], ex_jp = Ex[idx + sy];
        const float dhz = G.den_h[2][k];
        float hx = Hx[idx] + dt_mu0 * ((ez_c - ez_jp) * dhy + (ey_kp - ey_c) * dhz);
        float hy = Hy[idx] + dt_mu0 * ((ez_ip - ez_c) * dhx + (ex_c - ex_kp) * dhz);
        float hz = Hz[idx] + dt_mu0 * ((ey_c - ey_ip) * dhx + (ex_jp - ex_c) * dhy);
        if (lhx >= 0) {  // mxll_3D_mod.f90:585-620
            const long long p = lhx + (long long)G.L2 * ((j - 1) + (long long)L.ny * (k - 1));
            const float b = G.bH[0][i], c = G.cH[0][i];
            const float v0 = psi3<float, false>(b, G.psiH[0][0][p], c, ez_ip - ez_c, dr);
            const float v1 = psi3<float, false>(b, G.psiH[0][1][p], c, ey_c - ey_ip, dr);
            A.psiH_out[0][0][p] = v0;
            A.psiH_out[0][1][p] = v1;
            hy = hy + dt_mu0 * v0;
            hz = hz + dt_mu0 * v1;
        }
        if (lhy >= 0) {  // :622-657
            const long long p = (i - 1) + (long long)L.nx * (lhy + (long long)G.L2 * (k - 1));
            const float b = G.bH[1][j], c = G.cH[1][j];
            const float v0 = psi3<float, false>(b, G.psiH[1][0][p], c, ez_c - ez_jp, dr);
            const float v1 = psi3<float, false>(b, G.psiH[1][1][p], c, ex_jp - ex_c, dr);
            A.psiH_out[1][0][p] = v0;
            A.psiH_out[1][1][p] = v1;
            hx = hx + dt_mu0 * v0;
            hz = hz + dt_mu0 * v1;
        }
        const int lhz = G.lH[2][k];
        if (lhz >= 0) {  // :659-694
            const long long p = (i - 1) + (long long)L.nx * ((j - 1) + (long long)L.ny * lhz);
            const float b = G.bH[2][k], c = G.cH[2][k];
            const float v0 = psi3<float, false>(b, G.psiH[2][0][p], c, ey_kp - ey_c, dr);
            const float v1 = psi3<float, false>(b, G.psiH[2][1][p], c, ex_c - ex_kp, dr);
            A.psiH_out[2][0][p] = v0;
            A.psiH_out[2][1][p] = v1;
            hx = hx + dt_mu0 * v0;
            hy = hy + dt_mu0 * v1;
        }
        oHx[idx] = hx;
        oHy[idx] = hy;
        oHz[idx] = hz;
        // periodic ghost planes H(0) = H(n), as h3_tile writes them (read by the dispersive-cell
        // pass and the detectors)
        const bool gx = G.per[0] && i == L.nx, gy = G.per[1] && j == L.ny, gz = G.per[2] && k == L.nz;
        if (gx | gy | gz) {
            const long long ox = gx ? -(long long)L.nx : 0, oy = gy ? -(long long)L.ny * L.px : 0;
            const long long oz = gz ? -(long long)L.nz * L.pz : 0;
            if (gy) oHx[idx + oy] = hx;
            if (gz) oHx[idx + oz] = hx;
            if (gy && gz) oHx[idx + oy + oz] = hx;
            if (gx) oHy[idx + ox] = hy;
            if (gz) oHy[idx + oz] = hy;
            if (gx && gz) oHy[idx + ox + oz] = hy;
            if (gx) oHz[idx + ox] = hz;
            if (gy) oHz[idx + oy] = hz;
            if (gx && gy) oHz[idx + ox + oy] = hz;
        }
        // ---- new H of the neighbours the E update needs
        float hz_im = __shfl_up_sync(0xffffffffu, hz, 1), hy_im = __shfl_up_sync(0xffffffffu, hy, 1);
        if (tx == 0) {
            hz_im = f3_hnew<2>(A, G, i - 1, j, k);
            hy_im = f3_hnew<1>(A, G, i - 1, j, k);
        }
        const int pb = k & 1;
        sh_hz[pb][ty][tx] = hz;
        sh_hx[pb][ty][tx] = hx;
        __syncthreads();
        float hz_jm, hx_jm;
        if (ty > 0) {
            hz_jm = sh_hz[pb][ty - 1][tx];
            hx_jm = sh_hx[pb][ty - 1][tx];
        } else {
            hz_jm = f3_hnew<2>(A, G, i, j - 1, k);
            hx_jm = f3_hnew<0>(A, G, i, j - 1, k);
        }
        // ---- E_new(i, j, k): the expressions of e3_tile on the new H
        const float dez = G.den_e[2][k];
        const float rx = (hz - hz_jm) * dey + (hy_km - hy) * dez;
        const float ry = (hz_im - hz) * dex + (hx - hx_km) * dez;
        const float rz = (hy - hy_im) * dex + (hx_jm - hx) * dey;
        float ex = ex_c, ey = ey_c, ez = ez_c;
        if (bb_ij && k >= G.bb0[2] && k <= G.bb1[2]) {
            const long long b = (i - G.bb0[0]) + (long long)G.bbd[0] * ((j - G.bb0[1]) + (long long)G.bbd[1] * (k - G.bb0[2]));
            ex = plain_update<float>(ex, rx, G.mat[0][b], G);
            ey = plain_update<float>(ey, ry, G.mat[1][b], G);
            ez = plain_update<float>(ez, rz, G.mat[2][b], G);
        } else {
            ex = ex + dt_eps0 * rx;
            ey = ey + dt_eps0 * ry;
            ez = ez + dt_eps0 * rz;
        }
        if (lex >= 0) {  // mxll_3D_mod.f90:817-849
            const long long p = lex + (long long)G.L2 * ((j - 1) + (long long)L.ny * (k - 1));
            const float b = G.bE[0][i], c = G.cE[0][i];
            const float v0 = psi3<float, false>(b, G.psiE[0][0][p], c, hz_im - hz, dr);
            const float v1 = psi3<float, false>(b, G.psiE[0][1][p], c, hy - hy_im, dr);
            G.psiE[0][0][p] = v0;
            G.psiE[0][1][p] = v1;
            ey = ey + dt_eps0 * v0;
            ez = ez + dt_eps0 * v1;
        }
        if (ley >= 0) {  // :851-885
            const long long p = (i - 1) + (long long)L.nx * (ley + (long long)G.L2 * (k - 1));
            const float b = G.bE[1][j], c = G.cE[1][j];
            const float v0 = psi3<float, false>(b, G.psiE[1][0][p], c, hz - hz_jm, dr);
            const float v1 = psi3<float, false>(b, G.psiE[1][1][p], c, hx_jm - hx, dr);
            G.psiE[1][0][p] = v0;
            G.psiE[1][1][p] = v1;
            ex = ex + dt_eps0 * v0;
            ez = ez + dt_eps0 * v1;
        }
        const int lez = G.lE[2][k];
        if (lez >= 0) {  // :887-921
            const long long p = (i - 1) + (long long)L.nx * ((j - 1) + (long long)L.ny * lez);
            const float b = G.bE[2][k], c = G.cE[2][k];
            const float v0 = psi3<float, false>(b, G.psiE[2][0][p], c, hy_km - hy, dr);
            const float v1 = psi3<float, false>(b, G.psiE[2][1][p], c, hx - hx_km, dr);
            G.psiE[2][0][p] = v0;
            G.psiE[2][1][p] = v1;
            ex = ex + dt_eps0 * v0;
            ey = ey + dt_eps0 * v1;
        }
        oEx[idx] = ex;
        oEy[idx] = ey;
        oEz[idx] = ez;
        hx_km = hx;
        hy_km = hy;
        ex_c = ex_kp;
        ey_c = ey_kp;
    }
}

}  // namespace omx
