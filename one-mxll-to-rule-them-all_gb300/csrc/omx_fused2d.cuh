// omx_fused2d.cuh -- FP32 fused time step for 2D TMz: the H update (mxll_2D_mod.f90:469-552) and
// the E update (:661-748) of one step in a single pass over HBM.
//
// Each cell's Ez, Hx, Hy are read once and written once per step (6 words instead of the 9 of
// two half-step passes).  The pass reads the "in" buffers and writes the "out" buffers
// (ping-pong), because a block needs the new H of its left / lower neighbour cells, which it
// recomputes from the old values rather than waiting for the neighbouring block: recomputing
// from buffers nobody writes during the pass keeps blocks independent.  The CPML psi of H is
// ping-ponged for the same reason; psi of E and the ADE state are touched by their owner only.
//
// Work split: one thread owns 4 consecutive cells along x (float4 rows, 128-byte aligned) and
// marches JCH rows along y.  Hy_new(i-1) comes from the lower lane by a shuffle (lane 0
// recomputes it); Hx_new(j-1) is carried from the previous row (the first row recomputes it).
//
// Dispersive cells, sources and the emitter current are applied afterwards to the out buffer
// (k_ade_post, the source kernels, k_inject): they commute with the bulk update up to FP32
// rounding.  The host enables this path only when no dispersive cell lies in a CPML slab and no
// source point lies in a dispersive cell.
#pragma once
#include "omx_post.cuh"
#include "omx_stencil.cuh"
#include "omx_tma.cuh"

namespace omx {

// H of one TMz cell from old values (the reference's expressions; c prefolded with 1/dr).
__device__ __forceinline__ float fz_hx(float hx, float ez, float ez_jp, float dhy, float dt_mu0, int ly, float bh,
                                       float ch, const float *psi_in, float *psi_out, long long p)
{
    float h = hx + dt_mu0 * ((ez - ez_jp) * dhy);
    if (ly >= 0) {
        const float v = bh * psi_in[p] + ch * (ez - ez_jp);
        if (psi_out) psi_out[p] = v;
        h = h + dt_mu0 * v;
    }
    return h;
}
__device__ __forceinline__ float fz_hy(float hy, float ez, float ez_ip, float dhx, float dt_mu0, int lx, float bh,
                                       float ch, const float *psi_in, float *psi_out, long long p)
{
    float h = hy + dt_mu0 * ((ez_ip - ez) * dhx);
    if (lx >= 0) {
        const float v = bh * psi_in[p] + ch * (ez_ip - ez);
        if (psi_out) psi_out[p] = v;
        h = h + dt_mu0 * v;
    }
    return h;
}

// Rows j0..j1 of one column strip (128 threads x 4 cells = 512 columns).
template <bool XCPML>
__device__ __forceinline__ void fused_tmz_rows(const Fused2Args &A, const GridArgs<float> &G, int strip, int j0, int j1)
{
    const Lay &L = G.L;
    const int t = strip * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int ib = 1 + 4 * t;                 // first of this thread's 4 cells
    const bool active = ib <= L.nx;           // nx % 4 == 0 is required by the host
    const float dt_mu0 = G.dt_mu0, dt_eps0 = G.dt_eps0;
    const long long px = L.px;
    const int ibc = active ? ib : 1;          // lanes past nx only join the shuffles
    // per-column x factors: uniform 1/dr and no psi without an x CPML
    float dhx[4], dex[4], bhx[4], chx[4], bex[4], cex[4];
    int lhx[4], lex[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int i = XCPML ? min(ibc + q, L.nx) : 1;
        dhx[q] = G.den_h[0][i];
        dex[q] = G.den_e[0][i];
        lhx[q] = XCPML ? G.lH[0][i] : -1;
        lex[q] = XCPML ? G.lE[0][i] : -1;
        bhx[q] = XCPML ? G.bH[0][i] : 0.f;
        chx[q] = XCPML ? G.cH[0][i] : 0.f;
        bex[q] = XCPML ? G.bE[0][i] : 0.f;
        cex[q] = XCPML ? G.cE[0][i] : 0.f;
    }
    // left neighbour column (i = ib-1, or nx for a periodic wrap, or the PEC ghost); every
    // index below uses the clamped ibc so that lanes past nx stay inside the arrays
    const bool left_ghost = (ibc == 1) && !G.per[0];
    const int il = (ibc == 1) ? L.nx : ibc - 1;
    const float dhx_l = G.den_h[0][XCPML ? il : 1];
    const int lhx_l = XCPML ? G.lH[0][il] : -1;
    const float bhx_l = XCPML ? G.bH[0][il] : 0.f, chx_l = XCPML ? G.cH[0][il] : 0.f;
    // right neighbour for Ez(i+4): ib+4 (<= nx+1) or 1 when periodic at the last group
    const int iright = (ibc + 4 > L.nx && G.per[0]) ? 1 : ibc + 4;
    const bool bb_i = G.bbV > 0 && (ibc + 3 >= G.bb0[0] && ibc <= G.bb1[0]);
    const long long col = L.off + ibc;

    // Hx_new(i, j0-1): recomputed from old values (0 at a PEC ghost row)
    float hxp[4];
    {
        const int jm = j0 - 1;
        if (jm == 0 && !G.per[1]) {
#pragma unroll
            for (int q = 0; q < 4; ++q) hxp[q] = 0.f;
        } else {
            const int jr = (jm == 0) ? L.ny : jm;                     // periodic wrap
            const int jr1 = (jr == L.ny && G.per[1]) ? 1 : jr + 1;
            const float4 e0 = *reinterpret_cast<const float4 *>(A.ez_in + col + px * jr);
            const float4 e1 = *reinterpret_cast<const float4 *>(A.ez_in + col + px * jr1);
            const float4 h0 = *reinterpret_cast<const float4 *>(A.hx_in + col + px * jr);
            const float dhy = G.den_h[1][jr];
            const int ly = G.lH[1][jr];
            const float bh = G.bH[1][jr], ch = G.cH[1][jr];
            const long long pb = (ibc - 1) + (long long)L.nx * ly;
            hxp[0] = fz_hx(h0.x, e0.x, e1.x, dhy, dt_mu0, ly, bh, ch, A.psi_hxy_in, nullptr, pb + 0);
            hxp[1] = fz_hx(h0.y, e0.y, e1.y, dhy, dt_mu0, ly, bh, ch, A.psi_hxy_in, nullptr, pb + 1);
            hxp[2] = fz_hx(h0.z, e0.z, e1.z, dhy, dt_mu0, ly, bh, ch, A.psi_hxy_in, nullptr, pb + 2);
            hxp[3] = fz_hx(h0.w, e0.w, e1.w, dhy, dt_mu0, ly, bh, ch, A.psi_hxy_in, nullptr, pb + 3);
        }
    }
    // rows j and j+1 of Ez, row j of Hx / Hy in flight; the next row is fetched before the
    // current one is computed so two rows of loads overlap
    float4 ez_c = *reinterpret_cast<const float4 *>(A.ez_in + col + px * j0);
    int jn = (j0 == L.ny && G.per[1]) ? 1 : j0 + 1;
    float4 ez_n = *reinterpret_cast<const float4 *>(A.ez_in + col + px * jn);
    float4 hx_o = *reinterpret_cast<const float4 *>(A.hx_in + col + px * j0);
    float4 hy_o = *reinterpret_cast<const float4 *>(A.hy_in + col + px * j0);
    for (int j = j0; j <= j1; ++j) {
        const long long row = col + px * j;
        float4 ez_nn = ez_n, hx_on = hx_o, hy_on = hy_o;
        if (j < j1) {
            const int jnn = (j + 1 == L.ny && G.per[1]) ? 1 : j + 2;
            ez_nn = *reinterpret_cast<const float4 *>(A.ez_in + col + px * jnn);
            hx_on = *reinterpret_cast<const float4 *>(A.hx_in + row + px);
            hy_on = *reinterpret_cast<const float4 *>(A.hy_in + row + px);
        }
        // Ez(i+4, j): next lane's first element, or a load at the warp / row end
        float ez_r = __shfl_down_sync(0xffffffffu, ez_c.x, 1);
        if (lane == 31 || ibc + 4 > L.nx) ez_r = A.ez_in[L.off + iright + px * j];
        const float dhy = G.den_h[1][j], dey = G.den_e[1][j];
        const int ly = G.lH[1][j], lye = G.lE[1][j];
        const float bhy = G.bH[1][j], chy = G.cH[1][j], bey = G.bE[1][j], cey = G.cE[1][j];
        const float ez[5] = {ez_c.x, ez_c.y, ez_c.z, ez_c.w, ez_r};
        const float ezn[4] = {ez_n.x, ez_n.y, ez_n.z, ez_n.w};
        const float hxo[4] = {hx_o.x, hx_o.y, hx_o.z, hx_o.w};
        const float hyo[4] = {hy_o.x, hy_o.y, hy_o.z, hy_o.w};
        float hx[4], hy[4];
        const long long pby = (ibc - 1) + (long long)L.nx * ly;
        const long long pbx = (long long)G.L2 * (j - 1);
        float *const psx_out = active ? A.psi_hxy_out : nullptr;   // lanes past nx only join shuffles
        float *const psy_out = active ? A.psi_hyx_out : nullptr;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            hx[q] = fz_hx(hxo[q], ez[q], ezn[q], dhy, dt_mu0, ly, bhy, chy, A.psi_hxy_in, psx_out, pby + q);
            hy[q] = fz_hy(hyo[q], ez[q], ez[q + 1], dhx[q], dt_mu0, lhx[q], bhx[q], chx[q], A.psi_hyx_in,
                          psy_out, lhx[q] + pbx);
        }
        // Hy_new(i-1, j): previous lane's last cell, recomputed by lane 0
        float hy_l = __shfl_up_sync(0xffffffffu, hy[3], 1);
        if (active && (lane == 0 || ib == 1)) {
            if (left_ghost) {
                hy_l = 0.f;
            } else {
                const long long rl = L.off + il + px * j;
                // Ez(il+1) is this thread's first cell (or its periodic image)
                hy_l = fz_hy(A.hy_in[rl], A.ez_in[rl], ez[0], dhx_l, dt_mu0, lhx_l, bhx_l, chx_l, A.psi_hyx_in,
                             nullptr, lhx_l + pbx);
            }
        }
        if (active) {
            *reinterpret_cast<float4 *>(A.hx_out + row) = make_float4(hx[0], hx[1], hx[2], hx[3]);
            *reinterpret_cast<float4 *>(A.hy_out + row) = make_float4(hy[0], hy[1], hy[2], hy[3]);
            if (G.per[0] && ib + 3 == L.nx) A.hy_out[row + 3 - L.nx] = hy[3];            // Hy(0,j) = Hy(nx,j)
            if (G.per[1] && j == L.ny)
                *reinterpret_cast<float4 *>(A.hx_out + row - px * L.ny) = make_float4(hx[0], hx[1], hx[2], hx[3]);
            // E update of the 4 cells
            const bool bb = bb_i && j >= G.bb0[1] && j <= G.bb1[1];
            float eo[4];
            const float hyl[4] = {hy_l, hy[0], hy[1], hy[2]};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float dyh = hy[q] - hyl[q];
                const float dxh = hxp[q] - hx[q];
                const float r = dyh * dex[q] + dxh * dey;
                float e = ez[q];
                if (bb && ibc + q >= G.bb0[0] && ibc + q <= G.bb1[0]) {
                    const long long b = (ibc + q - G.bb0[0]) + (long long)G.bbd[0] * (j - G.bb0[1]);
                    e = plain_update<float>(e, r, G.mat[2][b], G);
                } else {
                    e = e + dt_eps0 * r;
                }
                if (XCPML && lex[q] >= 0) {
                    const long long p = lex[q] + pbx;
                    const float v = bex[q] * A.psi_ezx[p] + cex[q] * dyh;
                    A.psi_ezx[p] = v;
                    e = e + dt_eps0 * v;
                }
                if (lye >= 0) {
                    const long long p = (ibc + q - 1) + (long long)L.nx * lye;
                    const float v = bey * A.psi_ezy[p] + cey * dxh;
                    A.psi_ezy[p] = v;
                    e = e + dt_eps0 * v;
                }
                eo[q] = e;
            }
            *reinterpret_cast<float4 *>(A.ez_out + row) = make_float4(eo[0], eo[1], eo[2], eo[3]);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) hxp[q] = hx[q];
        ez_c = ez_n;
        ez_n = ez_nn;
        hx_o = hx_on;
        hy_o = hy_on;
    }
}

// Persistent launch: gridDim.x = SMs x resident blocks; the (strip, row) work is split into
// gridDim.x contiguous, equal ranges so every block marches about the same number of rows and
// no partial wave is left at the end.
template <bool XCPML>
__global__ void __launch_bounds__(128, 6) k_fused_tmz(Fused2Args A, GridArgs<float> G, int nstrip)
{
    if (G.step_inc && blockIdx.x == 0 && threadIdx.x == 0) *G.step_inc += 1;   // device-loop step counter
    const long long ny = G.L.ny;
    const long long total = (long long)nstrip * ny;
    long long r = total * blockIdx.x / gridDim.x;
    const long long r1 = total * (blockIdx.x + 1) / gridDim.x;
    while (r < r1) {
        const int strip = (int)(r / ny);
        const int j0 = (int)(r % ny) + 1;
        const int j1 = (int)min((long long)ny, (long long)j0 + (r1 - r) - 1);
        fused_tmz_rows<XCPML>(A, G, strip, j0, j1);
        r += j1 - j0 + 1;
    }
}

// ---------------------------------------------------------------------------------------------
// Register-tile variant: one block per (strip, tile of R rows), no persistent loop and no
// synchronisation of any kind.  Every thread issues all loads of its tile first (Ez of rows
// j0-1 .. j0+R, Hx of rows j0-1 .. j0+R-1, Hy of rows j0 .. j0+R-1, and the neighbour columns
// its edge lanes need), then computes the R rows from registers: up to 3R+3 float4 loads in
// flight per thread, the most memory-level parallelism a thread can carry.  The rows j0-1 and
// j0+R that a tile shares with its neighbours are read twice; consecutive blocks are vertically
// adjacent tiles of one strip, so the second read usually hits L2.  Same arithmetic on the same
// words as fused_tmz_rows.
template <bool XCPML, int R>
__global__ void __launch_bounds__(128, 4) k_fused_tmz_rt(Fused2Args A, GridArgs<float> G, int ntile)
{
    if (G.step_inc && blockIdx.x == 0 && threadIdx.x == 0) *G.step_inc += 1;   // device-loop step counter
    const Lay &L = G.L;
    const int tile = blockIdx.x % ntile, strip = blockIdx.x / ntile;
    const int j0 = 1 + R * tile;
    const int j1 = min(L.ny, j0 + R - 1);
    const float *__restrict__ ez_in = A.ez_in;
    const float *__restrict__ hx_in = A.hx_in;
    const float *__restrict__ hy_in = A.hy_in;
    float *__restrict__ ez_out = A.ez_out;
    float *__restrict__ hx_out = A.hx_out;
    float *__restrict__ hy_out = A.hy_out;
    const int t = strip * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int ib = 1 + 4 * t;
    const bool active = ib <= L.nx;
    const float dt_mu0 = G.dt_mu0, dt_eps0 = G.dt_eps0;
    const long long px = L.px;
    const int ibc = active ? ib : 1;
    const bool left_ghost = (ibc == 1) && !G.per[0];
    const int il = (ibc == 1) ? L.nx : ibc - 1;
    const int iright = (ibc + 4 > L.nx && G.per[0]) ? 1 : ibc + 4;
    const bool need_r = lane == 31 || ibc + 4 > L.nx;
    const bool need_l = active && (lane == 0 || ib == 1) && !left_ghost;
    const long long col = L.off + ibc;

    // ---- loads: every row of the tile (rows past j1 are not loaded)
    const int jm = j0 - 1;
    const bool has_m = !(jm == 0 && !G.per[1]);                 // Hx_new(j0-1) = 0 at a PEC ghost row
    const int jmr = (jm == 0) ? L.ny : jm;                      // periodic image of row 0
    float4 ezr[R + 2], hxr[R + 1], hyr[R];
    float ez_rt[R], hy_lt[R], ez_lt[R];
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    ezr[0] = has_m ? *reinterpret_cast<const float4 *>(ez_in + col + px * jmr) : z4;
    hxr[0] = has_m ? *reinterpret_cast<const float4 *>(hx_in + col + px * jmr) : z4;
#pragma unroll
    for (int r = 0; r <= R; ++r) {
        const int j = j0 + r;                                   // Ez rows j0 .. j1+1
        const int jj = (j == L.ny + 1 && G.per[1]) ? 1 : j;     // Ez(ny+1) = Ez(1)
        ezr[r + 1] = (j <= j1 + 1) ? *reinterpret_cast<const float4 *>(ez_in + col + px * jj) : z4;
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int j = j0 + r;
        const bool in = j <= j1;
        hxr[r + 1] = in ? *reinterpret_cast<const float4 *>(hx_in + col + px * j) : z4;
        hyr[r] = in ? *reinterpret_cast<const float4 *>(hy_in + col + px * j) : z4;
        ez_rt[r] = (in && need_r) ? ez_in[L.off + iright + px * j] : 0.f;
        hy_lt[r] = (in && need_l) ? hy_in[L.off + il + px * j] : 0.f;
        ez_lt[r] = (in && need_l) ? ez_in[L.off + il + px * j] : 0.f;
    }

    // ---- per-column x factors
    float dhx[4], dex[4], bhx[4], chx[4], bex[4], cex[4];
    int lhx[4], lex[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int i = XCPML ? min(ibc + q, L.nx) : 1;
        dhx[q] = G.den_h[0][i];
        dex[q] = G.den_e[0][i];
        lhx[q] = XCPML ? G.lH[0][i] : -1;
        lex[q] = XCPML ? G.lE[0][i] : -1;
        bhx[q] = XCPML ? G.bH[0][i] : 0.f;
        chx[q] = XCPML ? G.cH[0][i] : 0.f;
        bex[q] = XCPML ? G.bE[0][i] : 0.f;
        cex[q] = XCPML ? G.cE[0][i] : 0.f;
    }
    const float dhx_l = G.den_h[0][XCPML ? il : 1];
    const int lhx_l = XCPML ? G.lH[0][il] : -1;
    const float bhx_l = XCPML ? G.bH[0][il] : 0.f, chx_l = XCPML ? G.cH[0][il] : 0.f;
    const bool bb_i = G.bbV > 0 && (ibc + 3 >= G.bb0[0] && ibc <= G.bb1[0]);

    // ---- Hx_new(j0-1)
    float hxp[4] = {0.f, 0.f, 0.f, 0.f};
    if (has_m) {
        const float4 c0 = A.rowc[2 * jmr], c1 = A.rowc[2 * jmr + 1];
        const int ly = __float_as_int(c1.z);
        const long long pb = (ibc - 1) + (long long)L.nx * ly;
        const float4 e0 = ezr[0], e1 = ezr[1], h0 = hxr[0];
        hxp[0] = fz_hx(h0.x, e0.x, e1.x, c0.x, dt_mu0, ly, c0.z, c0.w, A.psi_hxy_in, nullptr, pb + 0);
        hxp[1] = fz_hx(h0.y, e0.y, e1.y, c0.x, dt_mu0, ly, c0.z, c0.w, A.psi_hxy_in, nullptr, pb + 1);
        hxp[2] = fz_hx(h0.z, e0.z, e1.z, c0.x, dt_mu0, ly, c0.z, c0.w, A.psi_hxy_in, nullptr, pb + 2);
        hxp[3] = fz_hx(h0.w, e0.w, e1.w, c0.x, dt_mu0, ly, c0.z, c0.w, A.psi_hxy_in, nullptr, pb + 3);
    }

    // ---- rows j0 .. j1 from registers
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int j = j0 + r;
        if (j > j1) break;                                      // uniform over the block
        const long long row = col + px * j;
        const float4 c0 = A.rowc[2 * j], c1 = A.rowc[2 * j + 1];
        const float dhy = c0.x, dey = c0.y, bhy = c0.z, chy = c0.w, bey = c1.x, cey = c1.y;
        const int ly = __float_as_int(c1.z), lye = __float_as_int(c1.w);
        const float4 ez_c = ezr[r + 1], ez_n = ezr[r + 2], hx_o = hxr[r + 1], hy_o = hyr[r];
        float ez_r = __shfl_down_sync(0xffffffffu, ez_c.x, 1);
        if (need_r) ez_r = ez_rt[r];
        const float ez[5] = {ez_c.x, ez_c.y, ez_c.z, ez_c.w, ez_r};
        const float ezn[4] = {ez_n.x, ez_n.y, ez_n.z, ez_n.w};
        const float hxo[4] = {hx_o.x, hx_o.y, hx_o.z, hx_o.w};
        const float hyo[4] = {hy_o.x, hy_o.y, hy_o.z, hy_o.w};
        float hx[4], hy[4];
        const long long pby = (ibc - 1) + (long long)L.nx * ly;
        const long long pbx = (long long)G.L2 * (j - 1);
        float *const psx_out = active ? A.psi_hxy_out : nullptr;
        float *const psy_out = active ? A.psi_hyx_out : nullptr;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            hx[q] = fz_hx(hxo[q], ez[q], ezn[q], dhy, dt_mu0, ly, bhy, chy, A.psi_hxy_in, psx_out, pby + q);
            hy[q] = fz_hy(hyo[q], ez[q], ez[q + 1], dhx[q], dt_mu0, lhx[q], bhx[q], chx[q], A.psi_hyx_in,
                          psy_out, lhx[q] + pbx);
        }
        float hy_l = __shfl_up_sync(0xffffffffu, hy[3], 1);
        if (active && (lane == 0 || ib == 1)) {
            hy_l = left_ghost ? 0.f
                              : fz_hy(hy_lt[r], ez_lt[r], ez[0], dhx_l, dt_mu0, lhx_l, bhx_l, chx_l, A.psi_hyx_in,
                                      nullptr, lhx_l + pbx);
        }
        if (active) {
            *reinterpret_cast<float4 *>(hx_out + row) = make_float4(hx[0], hx[1], hx[2], hx[3]);
            *reinterpret_cast<float4 *>(hy_out + row) = make_float4(hy[0], hy[1], hy[2], hy[3]);
            if (G.per[0] && ib + 3 == L.nx) hy_out[row + 3 - L.nx] = hy[3];            // Hy(0,j) = Hy(nx,j)
            if (G.per[1] && j == L.ny)
                *reinterpret_cast<float4 *>(hx_out + row - px * L.ny) = make_float4(hx[0], hx[1], hx[2], hx[3]);
            const bool bb = bb_i && j >= G.bb0[1] && j <= G.bb1[1];
            float eo[4];
            const float hyl[4] = {hy_l, hy[0], hy[1], hy[2]};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float dyh = hy[q] - hyl[q];
                const float dxh = hxp[q] - hx[q];
                const float rr = dyh * dex[q] + dxh * dey;
                float e = ez[q];
                if (bb && ibc + q >= G.bb0[0] && ibc + q <= G.bb1[0]) {
                    const long long b = (ibc + q - G.bb0[0]) + (long long)G.bbd[0] * (j - G.bb0[1]);
                    e = plain_update<float>(e, rr, G.mat[2][b], G);
                } else {
                    e = e + dt_eps0 * rr;
                }
                if (XCPML && lex[q] >= 0) {
                    const long long p = lex[q] + pbx;
                    const float v = bex[q] * A.psi_ezx[p] + cex[q] * dyh;
                    A.psi_ezx[p] = v;
                    e = e + dt_eps0 * v;
                }
                if (lye >= 0) {
                    const long long p = (ibc + q - 1) + (long long)L.nx * lye;
                    const float v = bey * A.psi_ezy[p] + cey * dxh;
                    A.psi_ezy[p] = v;
                    e = e + dt_eps0 * v;
                }
                eo[q] = e;
            }
            *reinterpret_cast<float4 *>(ez_out + row) = make_float4(eo[0], eo[1], eo[2], eo[3]);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) hxp[q] = hx[q];
    }
}

// ---------------------------------------------------------------------------------------------
// Bulk-copy variant: the same arithmetic, with the rows of Ez / Hx / Hy staged into shared memory
// by the TMA engine (cp.async.bulk, completion on an mbarrier per ring slot).  One thread issues
// the copies D-1 rows ahead of the row being computed, so the bytes in flight per SM no longer
// depend on registers.  A staged Ez / Hy row spans the strip's 512 columns plus 4 halo columns
// on each side (the left neighbour of the first cell, Ez(i+4) of the last thread); since every
// staged word is a copy of the same global address, results equal the register kernel's.
//
// Work items of one row segment (strip, rows j0..j1), in issue order:
//   item 0          row j0-1  Ez, Hx  (recomputes Hx_new(j0-1); nothing at a PEC ghost row)
//   items 1..n      rows j0..j1  Ez, Hx, Hy
//   item n+1        row j1+1  Ez only
// Step k (0..n) consumes items k and k+1, then releases item k (and item n+1 after step n).
constexpr int FZ_W = 512;                     // columns per strip chunk: 128 threads x 4 cells
// one ring slot for a strip of CH chunks: Ez / Hy with 4 halo columns each side, Hx without
template <int CH> struct FzStageT {
    float ez[FZ_W * CH + 8];                  // columns ib0-4 .. ib0+W+3
    float hy[FZ_W * CH + 8];
    float hx[FZ_W * CH];                      // columns ib0 .. ib0+W-1
};
using FzStage = FzStageT<1>;
static_assert(sizeof(FzStageT<1>) % 16 == 0 && sizeof(FzStageT<2>) % 16 == 0 && sizeof(FzStageT<4>) % 16 == 0 &&
                  (FZ_W + 8) % 4 == 0,
              "bulk copies need 16-byte aligned stage arrays");
constexpr long long FZ_WAIT_CYCLES = 2000000000LL;   // about one second at the SM clock

struct FzSeg {
    int strip, j0, j1;
};
__device__ __forceinline__ FzSeg fz_segment(long long r, long long r1, long long ny)
{
    FzSeg s;
    s.strip = (int)(r / ny);
    s.j0 = (int)(r % ny) + 1;
    s.j1 = (int)min(ny, (long long)s.j0 + (r1 - r) - 1);
    return s;
}

// Issue the copies of item k of segment S into stage st; completes on bar (one arrival).
template <int CH>
__device__ __forceinline__ void fz_issue(const Fused2Args &A, const GridArgs<float> &G, const FzSeg &S, int k,
                                         FzStageT<CH> *st, uint64_t *bar, uint64_t pol = 0)
{
    constexpr int W = FZ_W * CH;
    const Lay &L = G.L;
    const int ib0 = 1 + W * S.strip;
    const uint32_t ezb = 4u * (uint32_t)min(W + 8, L.nx - ib0 + 9);    // nx % 4 == 0: multiple of 16 B
    const uint32_t hxb = 4u * (uint32_t)min(W, L.nx - ib0 + 1);
    const int last = S.j1 - S.j0 + 2;
    int row = S.j0 - 1 + k;
    bool ld_ez = true, ld_hx = k < last, ld_hy = k > 0 && k < last;
    if (k == 0 && row == 0) {
        if (G.per[1]) row = L.ny;                                     // Hx_new(0) = Hx_new(ny)
        else ld_ez = ld_hx = false;                                   // PEC ghost row: Hx_new = 0
    }
    if (k == last && row == L.ny + 1 && G.per[1]) row = 1;            // Ez(ny+1) = Ez(1)
    const long long e0 = L.off + (ib0 - 4) + (long long)L.px * row;   // 16-byte aligned
    const long long h0 = L.off + ib0 + (long long)L.px * row;         // 128-byte aligned
    mbar_arrive_expect_tx(bar, (ld_ez ? ezb : 0u) + (ld_hx ? hxb : 0u) + (ld_hy ? ezb : 0u));
    if (pol) {
        if (ld_ez) bulk_g2s_hint(st->ez, A.ez_in + e0, ezb, bar, pol);
        if (ld_hx) bulk_g2s_hint(st->hx, A.hx_in + h0, hxb, bar, pol);
        if (ld_hy) bulk_g2s_hint(st->hy, A.hy_in + e0, ezb, bar, pol);
        return;
    }
    if (ld_ez) bulk_g2s(st->ez, A.ez_in + e0, ezb, bar);
    if (ld_hx) bulk_g2s(st->hx, A.hx_in + h0, hxb, bar);
    if (ld_hy) bulk_g2s(st->hy, A.hy_in + e0, ezb, bar);
}

template <bool XCPML, int D>
__global__ void __launch_bounds__(128, 6) k_fused_tmz_tma(Fused2Args A, GridArgs<float> G, int nstrip)
{
    extern __shared__ __align__(128) unsigned char fz_smem[];
    FzStage *stage = reinterpret_cast<FzStage *>(fz_smem);
    uint64_t *bar = reinterpret_cast<uint64_t *>(fz_smem + D * sizeof(FzStage));
    const Lay &L = G.L;
    const long long ny = L.ny;
    const long long total = (long long)nstrip * ny;
    const long long rb0 = total * blockIdx.x / gridDim.x;
    const long long rb1 = total * (blockIdx.x + 1) / gridDim.x;
    const int tl = threadIdx.x, lane = tl & 31;
    if (tl == 0) {
        if (G.step_inc && blockIdx.x == 0) *G.step_inc += 1;          // device-loop step counter
        for (int s = 0; s < D; ++s) mbar_init(&bar[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (rb0 >= rb1) return;

    // producer state (thread 0): the next item to issue and how many are issued / released
    long long pr = rb0;
    int pk = 0;
    int issued = 0, released = 0;             // items: rows + 2 per segment (fits an int)
    const uint64_t pol = tl == 0 ? l2_policy_evict_first() : 0;   // every row is read once per step
    auto issue_more = [&]() {
        while (pr < rb1 && issued < released + D) {
            const FzSeg S = fz_segment(pr, rb1, ny);
            const int slot = issued % D;
            fz_issue(A, G, S, pk, &stage[slot], &bar[slot], pol);
            ++issued;
            if (++pk == S.j1 - S.j0 + 3) {
                pk = 0;
                pr += S.j1 - S.j0 + 1;
            }
        }
    };
    if (tl == 0) issue_more();

    const float dt_mu0 = G.dt_mu0, dt_eps0 = G.dt_eps0;
    const long long px = L.px;
    bool fail = false;
    int m = 0;                                // index of the current segment's item 0
    for (long long r = rb0; r < rb1;) {
        const FzSeg S = fz_segment(r, rb1, ny);
        const int ib0 = 1 + FZ_W * S.strip;
        const int ib = ib0 + 4 * tl;
        const bool active = ib <= L.nx;
        const int ibc = active ? ib : 1;      // lanes past nx only join the shuffles
        float dhx[4], dex[4], bhx[4], chx[4], bex[4], cex[4];
        int lhx[4], lex[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = XCPML ? min(ibc + q, L.nx) : 1;
            dhx[q] = G.den_h[0][i];
            dex[q] = G.den_e[0][i];
            lhx[q] = XCPML ? G.lH[0][i] : -1;
            lex[q] = XCPML ? G.lE[0][i] : -1;
            bhx[q] = XCPML ? G.bH[0][i] : 0.f;
            chx[q] = XCPML ? G.cH[0][i] : 0.f;
            bex[q] = XCPML ? G.bE[0][i] : 0.f;
            cex[q] = XCPML ? G.cE[0][i] : 0.f;
        }
        const bool left_ghost = (ibc == 1) && !G.per[0];
        const int il = (ibc == 1) ? L.nx : ibc - 1;
        const float dhx_l = G.den_h[0][XCPML ? il : 1];
        const int lhx_l = XCPML ? G.lH[0][il] : -1;
        const float bhx_l = XCPML ? G.bH[0][il] : 0.f, chx_l = XCPML ? G.cH[0][il] : 0.f;
        const bool wrap_r = ibc + 4 > L.nx && G.per[0];
        const bool bb_i = G.bbV > 0 && (ibc + 3 >= G.bb0[0] && ibc <= G.bb1[0]);
        const long long col = L.off + ibc;
        const int n = S.j1 - S.j0 + 1;

        // step 0: Hx_new(j0-1) from items 0 and 1
        float hxp[4] = {0.f, 0.f, 0.f, 0.f};
        {
            const int s0 = m % D, s1 = (m + 1) % D;
            fail |= !mbar_wait_bounded(&bar[s0], (uint32_t)((m / D) & 1), FZ_WAIT_CYCLES);
            fail |= !mbar_wait_bounded(&bar[s1], (uint32_t)(((m + 1) / D) & 1), FZ_WAIT_CYCLES);
            fail = __any_sync(0xffffffffu, fail);   // warp-uniform, so the shuffles below stay converged
            const int jm = S.j0 - 1;
            if (!fail && !(jm == 0 && !G.per[1])) {
                const int jr = (jm == 0) ? L.ny : jm;
                const float4 e0 = *reinterpret_cast<const float4 *>(&stage[s0].ez[4 + 4 * tl]);
                const float4 e1 = *reinterpret_cast<const float4 *>(&stage[s1].ez[4 + 4 * tl]);
                const float4 h0 = *reinterpret_cast<const float4 *>(&stage[s0].hx[4 * tl]);
                const float dhy = G.den_h[1][jr];
                const int ly = G.lH[1][jr];
                const float bh = G.bH[1][jr], ch = G.cH[1][jr];
                const long long pb = (ibc - 1) + (long long)L.nx * ly;
                hxp[0] = fz_hx(h0.x, e0.x, e1.x, dhy, dt_mu0, ly, bh, ch, A.psi_hxy_in, nullptr, pb + 0);
                hxp[1] = fz_hx(h0.y, e0.y, e1.y, dhy, dt_mu0, ly, bh, ch, A.psi_hxy_in, nullptr, pb + 1);
                hxp[2] = fz_hx(h0.z, e0.z, e1.z, dhy, dt_mu0, ly, bh, ch, A.psi_hxy_in, nullptr, pb + 2);
                hxp[3] = fz_hx(h0.w, e0.w, e1.w, dhy, dt_mu0, ly, bh, ch, A.psi_hxy_in, nullptr, pb + 3);
            }
        }
        if (__syncthreads_or(fail)) goto drain;
        if (tl == 0) {
            ++released;
            issue_more();
        }

        // steps 1..n: row j = j0-1+k from items k (rows j) and k+1 (Ez of row j+1)
        for (int k = 1; k <= n; ++k) {
            const int j = S.j0 - 1 + k;
            const int sc = (m + k) % D, sn = (m + k + 1) % D;
            fail |= !mbar_wait_bounded(&bar[sn], (uint32_t)(((m + k + 1) / D) & 1), FZ_WAIT_CYCLES);
            fail = __any_sync(0xffffffffu, fail);
            if (!fail) {
                const FzStage &C = stage[sc];
                const float4 ez_c = *reinterpret_cast<const float4 *>(&C.ez[4 + 4 * tl]);
                const float4 ez_n = *reinterpret_cast<const float4 *>(&stage[sn].ez[4 + 4 * tl]);
                const float4 hx_o = *reinterpret_cast<const float4 *>(&C.hx[4 * tl]);
                const float4 hy_o = *reinterpret_cast<const float4 *>(&C.hy[4 + 4 * tl]);
                const long long row = col + px * j;
                // Ez(i+4, j): next lane's first cell, the staged halo, or Ez(1, j) when periodic
                float ez_r = __shfl_down_sync(0xffffffffu, ez_c.x, 1);
                if (lane == 31 || ibc + 4 > L.nx) ez_r = wrap_r ? A.ez_in[L.off + 1 + px * j] : C.ez[8 + 4 * tl];
                const float dhy = G.den_h[1][j], dey = G.den_e[1][j];
                const int ly = G.lH[1][j], lye = G.lE[1][j];
                const float bhy = G.bH[1][j], chy = G.cH[1][j], bey = G.bE[1][j], cey = G.cE[1][j];
                const float ez[5] = {ez_c.x, ez_c.y, ez_c.z, ez_c.w, ez_r};
                const float ezn[4] = {ez_n.x, ez_n.y, ez_n.z, ez_n.w};
                const float hxo[4] = {hx_o.x, hx_o.y, hx_o.z, hx_o.w};
                const float hyo[4] = {hy_o.x, hy_o.y, hy_o.z, hy_o.w};
                float hx[4], hy[4];
                const long long pby = (ibc - 1) + (long long)L.nx * ly;
                const long long pbx = (long long)G.L2 * (j - 1);
                float *const psx_out = active ? A.psi_hxy_out : nullptr;
                float *const psy_out = active ? A.psi_hyx_out : nullptr;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    hx[q] = fz_hx(hxo[q], ez[q], ezn[q], dhy, dt_mu0, ly, bhy, chy, A.psi_hxy_in, psx_out, pby + q);
                    hy[q] = fz_hy(hyo[q], ez[q], ez[q + 1], dhx[q], dt_mu0, lhx[q], bhx[q], chx[q], A.psi_hyx_in,
                                  psy_out, lhx[q] + pbx);
                }
                // Hy_new(i-1, j): previous lane's last cell; lane 0 recomputes it from the staged
                // left column, or from global memory for the periodic image of column 1
                float hy_l = __shfl_up_sync(0xffffffffu, hy[3], 1);
                if (active && (lane == 0 || ib == 1)) {
                    if (left_ghost) {
                        hy_l = 0.f;
                    } else if (ib == 1) {
                        const long long rl = L.off + il + px * j;
                        hy_l = fz_hy(A.hy_in[rl], A.ez_in[rl], ez[0], dhx_l, dt_mu0, lhx_l, bhx_l, chx_l,
                                     A.psi_hyx_in, nullptr, lhx_l + pbx);
                    } else {
                        hy_l = fz_hy(C.hy[3 + 4 * tl], C.ez[3 + 4 * tl], ez[0], dhx_l, dt_mu0, lhx_l, bhx_l, chx_l,
                                     A.psi_hyx_in, nullptr, lhx_l + pbx);
                    }
                }
                if (active) {
                    *reinterpret_cast<float4 *>(A.hx_out + row) = make_float4(hx[0], hx[1], hx[2], hx[3]);
                    *reinterpret_cast<float4 *>(A.hy_out + row) = make_float4(hy[0], hy[1], hy[2], hy[3]);
                    if (G.per[0] && ib + 3 == L.nx) A.hy_out[row + 3 - L.nx] = hy[3];            // Hy(0,j) = Hy(nx,j)
                    if (G.per[1] && j == L.ny)
                        *reinterpret_cast<float4 *>(A.hx_out + row - px * L.ny) = make_float4(hx[0], hx[1], hx[2], hx[3]);
                    const bool bb = bb_i && j >= G.bb0[1] && j <= G.bb1[1];
                    float eo[4];
                    const float hyl[4] = {hy_l, hy[0], hy[1], hy[2]};
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const float dyh = hy[q] - hyl[q];
                        const float dxh = hxp[q] - hx[q];
                        const float rr = dyh * dex[q] + dxh * dey;
                        float e = ez[q];
                        if (bb && ibc + q >= G.bb0[0] && ibc + q <= G.bb1[0]) {
                            const long long b = (ibc + q - G.bb0[0]) + (long long)G.bbd[0] * (j - G.bb0[1]);
                            e = plain_update<float>(e, rr, G.mat[2][b], G);
                        } else {
                            e = e + dt_eps0 * rr;
                        }
                        if (XCPML && lex[q] >= 0) {
                            const long long p = lex[q] + pbx;
                            const float v = bex[q] * A.psi_ezx[p] + cex[q] * dyh;
                            A.psi_ezx[p] = v;
                            e = e + dt_eps0 * v;
                        }
                        if (lye >= 0) {
                            const long long p = (ibc + q - 1) + (long long)L.nx * lye;
                            const float v = bey * A.psi_ezy[p] + cey * dxh;
                            A.psi_ezy[p] = v;
                            e = e + dt_eps0 * v;
                        }
                        eo[q] = e;
                    }
                    *reinterpret_cast<float4 *>(A.ez_out + row) = make_float4(eo[0], eo[1], eo[2], eo[3]);
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) hxp[q] = hx[q];
            }
            if (__syncthreads_or(fail)) goto drain;
            if (tl == 0) {
                released += (k == n) ? 2 : 1;     // the last step also frees the Ez-only item
                issue_more();
            }
        }
        m += n + 2;
        r += n;
    }
    return;
drain:
    // a wait ran out: flag it, give the copies still in flight a bounded time to land (so that no
    // copy writes this block's shared memory after it exits) and leave
    if (tl == 0) {
        atomicOr(A.err, 1);
        for (int q = released; q < issued; ++q)
            mbar_wait_bounded(&bar[q % D], (uint32_t)((q / D) & 1), FZ_WAIT_CYCLES);
    }
}

// ---------------------------------------------------------------------------------------------
// Warp-specialised bulk-copy variant.  Four consumer warps compute; a fifth warp issues the
// copies.  Every ring slot has a "full" barrier (one arrival plus the copy bytes) and an "empty"
// barrier (one arrival per consumer warp), so the consumer warps never wait for one another and
// the copy warp refills a slot as soon as the last consumer has read it: no block-wide barrier
// per row.  The copy warp follows the block's segments incrementally (no 64-bit division per
// item), and the y coefficients of a row come from the packed row table (two float4 loads).
// NW compute warps (4 or 8) and one copy warp per block; a strip chunk is 128 NW columns.
template <int NW, int CH> constexpr int fz_min_blocks() { return NW == 8 ? 3 : (CH == 1 ? 5 : 4); }

template <bool XCPML, int D, int CH, int NW>
__global__ void __launch_bounds__(32 * (NW + 1), (fz_min_blocks<NW, CH>())) k_fused_tmz_ws(Fused2Args A,
                                                                                      GridArgs<float> G, int nstrip)
{
    constexpr int FZ_CONSUMERS = NW;
    constexpr int WC = 128 * NW;               // columns per chunk: NW warps x 32 lanes x 4 cells
    constexpr int SW = WC * CH / FZ_W;         // the stage type's width in units of 512 columns
    constexpr int W = WC * CH;                 // strip width: each thread owns CH chunks of 4 cells
    extern __shared__ __align__(128) unsigned char fz_smem[];
    FzStageT<SW> *stage = reinterpret_cast<FzStageT<SW> *>(fz_smem);
    uint64_t *full = reinterpret_cast<uint64_t *>(fz_smem + D * sizeof(FzStageT<SW>));
    uint64_t *empty = full + D;
    const Lay &L = G.L;
    const long long ny = L.ny;
    const long long total = (long long)nstrip * ny;
    const long long rb0 = total * blockIdx.x / gridDim.x;
    const long long rb1 = total * (blockIdx.x + 1) / gridDim.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        if (G.step_inc && blockIdx.x == 0) *G.step_inc += 1;          // device-loop step counter
        for (int s = 0; s < D; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], FZ_CONSUMERS);
        }
        mbar_fence_init();
    }
    __syncthreads();
    if (rb0 >= rb1) return;

    if (warp == FZ_CONSUMERS) {
        // ---- copy warp: lane 0 issues every item of the block's range in order
        if (lane != 0) return;
        FzSeg S = fz_segment(rb0, rb1, ny);
        long long r = rb0;
        int k = 0, q = 0;
        bool ok = true;
        const uint64_t pol = l2_policy_evict_first();   // every row is read once per step
        for (;;) {
            const int slot = q % D;
            // item q reuses the slot of item q-D: wait until every consumer warp released it
            if (q >= D && !mbar_wait_bounded(&empty[slot], (uint32_t)(((q / D) - 1) & 1), FZ_WAIT_CYCLES)) {
                ok = false;
                break;
            }
            fz_issue<SW>(A, G, S, k, &stage[slot], &full[slot], pol);
            ++q;
            if (++k == S.j1 - S.j0 + 3) {
                k = 0;
                r += S.j1 - S.j0 + 1;
                if (r >= rb1) break;
                // a segment ends at its strip's last row or at the range end: the next one
                // starts at row 1 of the next strip
                S.strip += 1;
                S.j0 = 1;
                S.j1 = (int)min(ny, rb1 - r);
            }
        }
        if (!ok) {
            // a consumer stopped: flag it, let the copies in flight land, leave
            atomicOr(A.err, 1);
            for (int p = max(0, q - D); p < q; ++p)
                mbar_wait_bounded(&full[p % D], (uint32_t)((p / D) & 1), FZ_WAIT_CYCLES);
        }
        return;
    }

    // ---- consumer warps: the arithmetic of k_fused_tmz_tma, rows from the ring; chunk c of a
    // thread covers columns ib0 + 512 c + 4 tl .. +3, at stage offset 512 c
    const int tl = threadIdx.x;
    const float dt_mu0 = G.dt_mu0, dt_eps0 = G.dt_eps0;
    const long long px = L.px;
    int m = 0;                                // index of the current segment's item 0
    for (long long r = rb0; r < rb1;) {
        const FzSeg S = fz_segment(r, rb1, ny);
        const int ib0 = 1 + W * S.strip;
        bool active[CH], left_ghost[CH], wrap_r[CH], bb_i[CH];
        int ibc[CH], lhx_l[CH];
        float dhx_l[CH], bhx_l[CH], chx_l[CH];
        float dhx[CH][4], dex[CH][4], bhx[CH][4], chx[CH][4], bex[CH][4], cex[CH][4];
        int lhx[CH][4], lex[CH][4];
#pragma unroll
        for (int c = 0; c < CH; ++c) {
            const int ib = ib0 + WC * c + 4 * tl;
            active[c] = ib <= L.nx;
            ibc[c] = active[c] ? ib : 1;      // lanes past nx only join the shuffles
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int i = XCPML ? min(ibc[c] + q, L.nx) : 1;
                dhx[c][q] = G.den_h[0][i];
                dex[c][q] = G.den_e[0][i];
                lhx[c][q] = XCPML ? G.lH[0][i] : -1;
                lex[c][q] = XCPML ? G.lE[0][i] : -1;
                bhx[c][q] = XCPML ? G.bH[0][i] : 0.f;
                chx[c][q] = XCPML ? G.cH[0][i] : 0.f;
                bex[c][q] = XCPML ? G.bE[0][i] : 0.f;
                cex[c][q] = XCPML ? G.cE[0][i] : 0.f;
            }
            left_ghost[c] = (ibc[c] == 1) && !G.per[0];
            const int il = (ibc[c] == 1) ? L.nx : ibc[c] - 1;
            dhx_l[c] = G.den_h[0][XCPML ? il : 1];
            lhx_l[c] = XCPML ? G.lH[0][il] : -1;
            bhx_l[c] = XCPML ? G.bH[0][il] : 0.f;
            chx_l[c] = XCPML ? G.cH[0][il] : 0.f;
            wrap_r[c] = ibc[c] + 4 > L.nx && G.per[0];
            bb_i[c] = G.bbV > 0 && (ibc[c] + 3 >= G.bb0[0] && ibc[c] <= G.bb1[0]);
        }
        const int n = S.j1 - S.j0 + 1;
        bool fail = false;

        // step 0: Hx_new(j0-1) from items 0 and 1
        float hxp[CH][4];
#pragma unroll
        for (int c = 0; c < CH; ++c)
#pragma unroll
            for (int q = 0; q < 4; ++q) hxp[c][q] = 0.f;
        {
            const int s0 = m % D, s1 = (m + 1) % D;
            fail |= !mbar_wait_bounded(&full[s0], (uint32_t)((m / D) & 1), FZ_WAIT_CYCLES);
            fail |= !mbar_wait_bounded(&full[s1], (uint32_t)(((m + 1) / D) & 1), FZ_WAIT_CYCLES);
            fail = __any_sync(0xffffffffu, fail);
            if (fail) {
                if (lane == 0) atomicOr(A.err, 1);
                return;
            }
            const int jm = S.j0 - 1;
            if (!(jm == 0 && !G.per[1])) {
                const int jr = (jm == 0) ? L.ny : jm;
                const float4 c0 = A.rowc[2 * jr], c1 = A.rowc[2 * jr + 1];
                const int ly = __float_as_int(c1.z);
#pragma unroll
                for (int c = 0; c < CH; ++c) {
                    const int so = WC * c + 4 * tl;
                    const float4 e0 = *reinterpret_cast<const float4 *>(&stage[s0].ez[4 + so]);
                    const float4 e1 = *reinterpret_cast<const float4 *>(&stage[s1].ez[4 + so]);
                    const float4 h0 = *reinterpret_cast<const float4 *>(&stage[s0].hx[so]);
                    const long long pb = (ibc[c] - 1) + (long long)L.nx * ly;
                    hxp[c][0] = fz_hx(h0.x, e0.x, e1.x, c0.x, dt_mu0, ly, c0.z, c0.w, A.psi_hxy_in, nullptr, pb + 0);
                    hxp[c][1] = fz_hx(h0.y, e0.y, e1.y, c0.x, dt_mu0, ly, c0.z, c0.w, A.psi_hxy_in, nullptr, pb + 1);
                    hxp[c][2] = fz_hx(h0.z, e0.z, e1.z, c0.x, dt_mu0, ly, c0.z, c0.w, A.psi_hxy_in, nullptr, pb + 2);
                    hxp[c][3] = fz_hx(h0.w, e0.w, e1.w, c0.x, dt_mu0, ly, c0.z, c0.w, A.psi_hxy_in, nullptr, pb + 3);
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[s0]);                // item 0 is done
        }

        // steps 1..n: row j = j0-1+k from items k (row j) and k+1 (Ez of row j+1).  The global
        // words a row needs besides the ring (its y coefficients, and the periodic images of
        // columns 1 and nx at the strip ends) are loaded one row ahead, so their latency hides
        // behind the previous row's arithmetic.
        float4 c0n = A.rowc[2 * S.j0], c1n = A.rowc[2 * S.j0 + 1];
        float wr_n[CH], hyw_n[CH], ezw_n[CH];
#pragma unroll
        for (int c = 0; c < CH; ++c) {
            const bool wl = active[c] && ibc[c] == 1 && !left_ghost[c];
            wr_n[c] = wrap_r[c] ? A.ez_in[L.off + 1 + px * S.j0] : 0.f;
            hyw_n[c] = wl ? A.hy_in[L.off + L.nx + px * S.j0] : 0.f;
            ezw_n[c] = wl ? A.ez_in[L.off + L.nx + px * S.j0] : 0.f;
        }
        for (int k = 1; k <= n; ++k) {
            const int j = S.j0 - 1 + k;
            const int sc = (m + k) % D, sn = (m + k + 1) % D;
            const float4 c0 = c0n, c1 = c1n;
            float wr[CH], hyw[CH], ezw[CH];
#pragma unroll
            for (int c = 0; c < CH; ++c) {
                wr[c] = wr_n[c];
                hyw[c] = hyw_n[c];
                ezw[c] = ezw_n[c];
            }
            if (k < n) {
                c0n = A.rowc[2 * (j + 1)];
                c1n = A.rowc[2 * (j + 1) + 1];
#pragma unroll
                for (int c = 0; c < CH; ++c) {
                    const bool wl = active[c] && ibc[c] == 1 && !left_ghost[c];
                    if (wrap_r[c]) wr_n[c] = A.ez_in[L.off + 1 + px * (j + 1)];
                    if (wl) {
                        hyw_n[c] = A.hy_in[L.off + L.nx + px * (j + 1)];
                        ezw_n[c] = A.ez_in[L.off + L.nx + px * (j + 1)];
                    }
                }
            }
            fail = !mbar_wait_bounded(&full[sn], (uint32_t)(((m + k + 1) / D) & 1), FZ_WAIT_CYCLES);
            fail = __any_sync(0xffffffffu, fail);
            if (fail) {
                if (lane == 0) atomicOr(A.err, 1);
                return;
            }
            const FzStageT<SW> &C = stage[sc];
            const float dhy = c0.x, dey = c0.y, bhy = c0.z, chy = c0.w, bey = c1.x, cey = c1.y;
            const int ly = __float_as_int(c1.z), lye = __float_as_int(c1.w);
            const long long pbx = (long long)G.L2 * (j - 1);
            float hx[CH][4], hy[CH][4], hy_l[CH], ez[CH][5];
#pragma unroll
            for (int c = 0; c < CH; ++c) {
                const int so = WC * c + 4 * tl;
                const float4 ez_c = *reinterpret_cast<const float4 *>(&C.ez[4 + so]);
                const float4 ez_n = *reinterpret_cast<const float4 *>(&stage[sn].ez[4 + so]);
                const float4 hx_o = *reinterpret_cast<const float4 *>(&C.hx[so]);
                const float4 hy_o = *reinterpret_cast<const float4 *>(&C.hy[4 + so]);
                float ez_r = __shfl_down_sync(0xffffffffu, ez_c.x, 1);
                if (lane == 31 || ibc[c] + 4 > L.nx) ez_r = wrap_r[c] ? wr[c] : C.ez[8 + so];
                ez[c][0] = ez_c.x;
                ez[c][1] = ez_c.y;
                ez[c][2] = ez_c.z;
                ez[c][3] = ez_c.w;
                ez[c][4] = ez_r;
                const float ezn[4] = {ez_n.x, ez_n.y, ez_n.z, ez_n.w};
                const float hxo[4] = {hx_o.x, hx_o.y, hx_o.z, hx_o.w};
                const float hyo[4] = {hy_o.x, hy_o.y, hy_o.z, hy_o.w};
                const long long pby = (ibc[c] - 1) + (long long)L.nx * ly;
                float *const psx_out = active[c] ? A.psi_hxy_out : nullptr;
                float *const psy_out = active[c] ? A.psi_hyx_out : nullptr;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    hx[c][q] = fz_hx(hxo[q], ez[c][q], ezn[q], dhy, dt_mu0, ly, bhy, chy, A.psi_hxy_in, psx_out, pby + q);
                    hy[c][q] = fz_hy(hyo[q], ez[c][q], ez[c][q + 1], dhx[c][q], dt_mu0, lhx[c][q], bhx[c][q], chx[c][q],
                                     A.psi_hyx_in, psy_out, lhx[c][q] + pbx);
                }
                // Hy_new(i-1, j): previous lane's last cell; lane 0 recomputes it from the staged
                // left column, or from global memory for the periodic image of column 1
                hy_l[c] = __shfl_up_sync(0xffffffffu, hy[c][3], 1);
                const int ib = ibc[c];
                if (active[c] && (lane == 0 || ib == 1)) {
                    if (left_ghost[c]) {
                        hy_l[c] = 0.f;
                    } else if (ib == 1) {
                        hy_l[c] = fz_hy(hyw[c], ezw[c], ez[c][0], dhx_l[c], dt_mu0, lhx_l[c], bhx_l[c], chx_l[c],
                                        A.psi_hyx_in, nullptr, lhx_l[c] + pbx);
                    } else {
                        hy_l[c] = fz_hy(C.hy[3 + so], C.ez[3 + so], ez[c][0], dhx_l[c], dt_mu0, lhx_l[c], bhx_l[c],
                                        chx_l[c], A.psi_hyx_in, nullptr, lhx_l[c] + pbx);
                    }
                }
            }
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&empty[sc]);                           // row j is read
                if (k == n) mbar_arrive(&empty[sn]);               // and the Ez-only item after it
            }
#pragma unroll
            for (int c = 0; c < CH; ++c) {
                if (active[c]) {
                    const long long row = L.off + ibc[c] + px * j;
                    __stcs(reinterpret_cast<float4 *>(A.hx_out + row), make_float4(hx[c][0], hx[c][1], hx[c][2], hx[c][3]));
                    __stcs(reinterpret_cast<float4 *>(A.hy_out + row), make_float4(hy[c][0], hy[c][1], hy[c][2], hy[c][3]));
                    if (G.per[0] && ibc[c] + 3 == L.nx) A.hy_out[row + 3 - L.nx] = hy[c][3];   // Hy(0,j) = Hy(nx,j)
                    if (G.per[1] && j == L.ny)
                        *reinterpret_cast<float4 *>(A.hx_out + row - px * L.ny) =
                            make_float4(hx[c][0], hx[c][1], hx[c][2], hx[c][3]);
                    const bool bb = bb_i[c] && j >= G.bb0[1] && j <= G.bb1[1];
                    float eo[4];
                    const float hyl[4] = {hy_l[c], hy[c][0], hy[c][1], hy[c][2]};
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const float dyh = hy[c][q] - hyl[q];
                        const float dxh = hxp[c][q] - hx[c][q];
                        const float rr = dyh * dex[c][q] + dxh * dey;
                        float e = ez[c][q];
                        const int ic = ibc[c] + q;
                        if (bb && ic >= G.bb0[0] && ic <= G.bb1[0]) {
                            const long long b = (ic - G.bb0[0]) + (long long)G.bbd[0] * (j - G.bb0[1]);
                            e = plain_update<float>(e, rr, G.mat[2][b], G);
                        } else {
                            e = e + dt_eps0 * rr;
                        }
                        if (XCPML && lex[c][q] >= 0) {
                            const long long p = lex[c][q] + pbx;
                            const float v = bex[c][q] * A.psi_ezx[p] + cex[c][q] * dyh;
                            A.psi_ezx[p] = v;
                            e = e + dt_eps0 * v;
                        }
                        if (lye >= 0) {
                            const long long p = (ic - 1) + (long long)L.nx * lye;
                            const float v = bey * A.psi_ezy[p] + cey * dxh;
                            A.psi_ezy[p] = v;
                            e = e + dt_eps0 * v;
                        }
                        eo[q] = e;
                    }
                    __stcs(reinterpret_cast<float4 *>(A.ez_out + row), make_float4(eo[0], eo[1], eo[2], eo[3]));
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) hxp[c][q] = hx[c][q];
            }
        }
        m += n + 2;
        r += n;
    }
}

// Dispersive cells after the fused pass: E_out = ADE(E_in, curl H_out) (no CPML term: the host
// keeps dispersive cells out of the CPML slabs on this path).
__device__ __forceinline__ void ade_post_cell(const FieldPtrs<float> &Fin, const FieldPtrs<float> &Fout,
                                              const GridArgs<float> &G, int q)
{
    const int4 en = G.ade_ent[q];
    const int b = G.ade_b[q];
    const int c = en.w;
    const float rot = curl_h<float>(Fout, G, c, en.x, en.y, en.z);
    const Lay &L = G.L;
    const long long idx = L.off + en.x + (long long)L.px * en.y + L.pz * en.z;
    const ClsR<float> cl = G.cls[G.mat[c][b]];
    Fout.f[c][idx] = ade_update<float>(Fin.f[c][idx], rot, cl, c, b, G);
}
__global__ void k_ade_post(FieldPtrs<float> Fin, FieldPtrs<float> Fout, GridArgs<float> G)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < G.ade_n) ade_post_cell(Fin, Fout, G, q);
}

// Dispersive cells, the plane source and the emitter current after the fused pass in one launch:
// the first nb_ade blocks take the dispersive cells, the next nb_plane the plane's cells, the
// rest the emitter-current points.  The lists write disjoint E words (the host checks), and each
// word gets the operation of its separate kernel, so the result is the same.
__global__ void __launch_bounds__(128) k_post_fused(FieldPtrs<float> Fin, FieldPtrs<float> Fout, GridArgs<float> G,
                                                    PostArgs Q)
{
    int b = blockIdx.x;
    const int t = threadIdx.x;
    if (b < Q.nb_ade) {
        const int q = b * 128 + t;
        if (q < G.ade_n) ade_post_cell(Fin, Fout, G, q);
        return;
    }
    b -= Q.nb_ade;
    if (b < Q.nb_plane) {
        const double amp = sp_get(Q.amp);
        const int q = b * 128 + t;
        if (amp != 0.0 && q < Q.plane_cells) plane_point<float>(Fout, G.L, Q.P, amp, q % Q.plane_n0, q / Q.plane_n0);
        return;
    }
    b -= Q.nb_plane;
    const int q = b * 128 + t;
    if (q < Q.I.n) inject_point<float>(Fout, Q.J, Q.I, sp_get(Q.time) - sp_get(Q.tskip), Q.dt_eps0, q);
}

}  // namespace omx
