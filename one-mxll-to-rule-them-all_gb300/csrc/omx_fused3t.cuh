// omx_fused3t.cuh -- FP32 single-pass 3D time step with the field planes staged in shared memory
// by the tensor-memory accelerator: the H update (mxll_3D_mod.f90:505-696), the E update with
// its Drude / Drude-Lorentz ADE (:700-923, classical_medium_mod.f90:773-833), both CPML
// recursions and a plane soft source in one pass over HBM.
//
// Every cell's six field words are read once and written once per step (12 words instead of the
// 18 of two half-step passes), and the dispersive cells are updated in the same pass (their ADE
// state is read and written once).  The pass reads the "in" buffer set and writes the "out" set
// (ping-pong, H psi included), so that the new H a cell's E update needs at i-1 and j-1 can be
// recomputed by this block from buffers nobody writes during the pass.
//
// Block: a 32 x TY tile of (i, j) columns marching kch planes along k.
//   * a copy warp (one lane) loads, per plane, the 6 components over x = i0-4 .. i0+35 (the box
//     starts on a 16-byte boundary) and y = j0-1 .. j0+TY into a ring of D plane slots, one
//     3D tensor-map copy per component, completing on the slot's "full" mbarrier; it refills a
//     slot once its "empty" mbarrier has an arrival from every compute warp;
//   * TY compute warps own one row of 32 cells each: new H from the staged E of planes k and k+1,
//     into shared memory; then new E from the staged old E, the new H of (i-1), (j-1) from shared
//     memory and the new H of plane k-1 from registers;
//   * a halo warp computes the new H of row j0-1 (Hz, Hx) and column i0-1 (Hz, Hy) of the tile.
// One named barrier per plane (the compute and halo warps) separates the two halves; the new-H
// tile is double-buffered by plane parity.  The same device function computes a component's new
// H for its owner and for a neighbouring block's halo, with explicit round-to-nearest operations,
// so both get the same bits.
//
// Every copy starts inside the tensor on a 16-byte boundary (the box may reach past a dimension,
// where the copy engine fills zeros) and every barrier wait is bounded: a wait that runs out sets
// bit 0 of the error word, all consumer warps leave the plane loop together (the barrier also
// votes), and the copy warp lets its copies in flight land before it leaves.
//
// Eligibility (host): FP32, x and y not periodic (the staged halo then holds the PEC ghosts),
// no point of a radial source in a dispersive cell (the radial sources and the emitter current
// are added after the pass).  Any nx, ny: tiles past the edge compute on zero-filled staging and
// write nothing.
#pragma once
#include <cuda.h>
#include "omx_post.cuh"
#include "omx_stencil.cuh"
#include "omx_tma.cuh"

namespace omx {

constexpr int F3T_BX = 40;    // staged box width: x from i0-4 (16-byte aligned) to i0+35
constexpr int F3T_D = 4;      // ring depth in planes
constexpr long long F3T_WAIT_CYCLES = 2000000000LL;   // about one second at the SM clock

// bytes reserved for a grid's GridArgs copy in the batched kernel's shared memory
constexpr int F3T_ARGB = (int)((sizeof(GridArgs<float>) + 15) / 16 * 16);

template <int TY> struct F3tShape {
    static constexpr int BY = TY + 2;                          // staged rows j0-1 .. j0+TY
    static constexpr int BOXF = F3T_BX * BY;                   // floats per staged box
    static constexpr int BOXB = (BOXF * 4 + 127) / 128 * 128;  // bytes per box slot (128-byte aligned)
    static constexpr int SLOTB = 6 * BOXB;                     // one plane: Ex, Ey, Ez, Hx, Hy, Hz
    static constexpr int HNF = (TY + 1) * 33;                  // new-H tile incl. column i0-1 and row j0-1
    static constexpr int SMEM = F3T_D * SLOTB + 2 * 3 * HNF * 4 + 2 * F3T_D * 8;
    // with the copy of the grid's arguments (GridArgs, Fused3Args) that the kernels read
    // with the copy of the grid's arguments (GridArgs, Fused3Args) that the kernels read
    static constexpr int SMEM_BATCH = SMEM + F3T_ARGB + (int)((sizeof(Fused3Args) + 15) / 16 * 16);
    static constexpr int THREADS = 32 * (TY + 2);
};

__device__ __forceinline__ void tma_load_3d(void *dst, const void *tmap, int x, int y, int z, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// barrier `id` over `n` threads that also returns whether any of them passed pred = true
__device__ __forceinline__ bool bar_any(int id, int n, bool pred)
{
    uint32_t r;
    asm volatile(
        "{\n"
        " .reg .pred p, q;\n"
        " setp.ne.u32 q, %1, 0;\n"
        " bar.red.or.pred p, %2, %3, q;\n"
        " selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(r)
        : "r"((uint32_t)pred), "r"(id), "r"(n)
        : "memory");
    return r != 0;
}

// One CPML psi step (FP32 path: 1/dr folded into c) and its H / E contribution.
__device__ __forceinline__ float f3t_psi(float b, float psi, float c, float d)
{
    return __fmaf_rn(b, psi, __fmul_rn(c, d));
}

// New H components (h3_tile's expressions, the CPML faces in the reference's order) from the
// staged neighbourhood.  pm: 0 no psi access (a cell past the grid edge, whose value nobody
// uses), 1 read the in set's psi (a halo cell, or the plane before the first), 2 read and write
// the out set's psi (the owner).
__device__ __forceinline__ float f3t_hx(float hx, float ez_c, float ez_jp, float ey_c, float ey_kp, float dhy,
                                        float dhz, float dt_mu0, int ly, int lz, const GridArgs<float> &G,
                                        const Fused3Args &A, int i, int j, int kk, int pm)
{
    float h = __fmaf_rn(dt_mu0, __fmaf_rn(ey_kp - ey_c, dhz, __fmul_rn(ez_c - ez_jp, dhy)), hx);
    const Lay &L = G.L;
    if (ly >= 0 && pm) {   // mxll_3D_mod.f90:622-657
        const int p = (i - 1) + L.nx * (ly + G.L2 * (kk - 1));
        const float v = f3t_psi(G.bH[1][j], G.psiH[1][0][p], G.cH[1][j], ez_c - ez_jp);
        if (pm == 2) A.psiH_out[1][0][p] = v;
        h = __fmaf_rn(dt_mu0, v, h);
    }
    if (lz >= 0 && pm) {   // :659-694
        const int p = (i - 1) + L.nx * ((j - 1) + L.ny * lz);
        const float v = f3t_psi(G.bH[2][kk], G.psiH[2][0][p], G.cH[2][kk], ey_kp - ey_c);
        if (pm == 2) A.psiH_out[2][0][p] = v;
        h = __fmaf_rn(dt_mu0, v, h);
    }
    return h;
}
__device__ __forceinline__ float f3t_hy(float hy, float ez_c, float ez_ip, float ex_c, float ex_kp, float dhx,
                                        float dhz, float dt_mu0, int lx, int lz, const GridArgs<float> &G,
                                        const Fused3Args &A, int i, int j, int kk, int pm)
{
    float h = __fmaf_rn(dt_mu0, __fmaf_rn(ex_c - ex_kp, dhz, __fmul_rn(ez_ip - ez_c, dhx)), hy);
    const Lay &L = G.L;
    if (lx >= 0 && pm) {   // mxll_3D_mod.f90:585-620
        const int p = lx + G.L2 * ((j - 1) + L.ny * (kk - 1));
        const float v = f3t_psi(G.bH[0][i], G.psiH[0][0][p], G.cH[0][i], ez_ip - ez_c);
        if (pm == 2) A.psiH_out[0][0][p] = v;
        h = __fmaf_rn(dt_mu0, v, h);
    }
    if (lz >= 0 && pm) {
        const int p = (i - 1) + L.nx * ((j - 1) + L.ny * lz);
        const float v = f3t_psi(G.bH[2][kk], G.psiH[2][1][p], G.cH[2][kk], ex_c - ex_kp);
        if (pm == 2) A.psiH_out[2][1][p] = v;
        h = __fmaf_rn(dt_mu0, v, h);
    }
    return h;
}
__device__ __forceinline__ float f3t_hz(float hz, float ey_c, float ey_ip, float ex_c, float ex_jp, float dhx,
                                        float dhy, float dt_mu0, int lx, int ly, const GridArgs<float> &G,
                                        const Fused3Args &A, int i, int j, int kk, int pm)
{
    float h = __fmaf_rn(dt_mu0, __fmaf_rn(ex_jp - ex_c, dhy, __fmul_rn(ey_c - ey_ip, dhx)), hz);
    const Lay &L = G.L;
    if (lx >= 0 && pm) {
        const int p = lx + G.L2 * ((j - 1) + L.ny * (kk - 1));
        const float v = f3t_psi(G.bH[0][i], G.psiH[0][1][p], G.cH[0][i], ey_c - ey_ip);
        if (pm == 2) A.psiH_out[0][1][p] = v;
        h = __fmaf_rn(dt_mu0, v, h);
    }
    if (ly >= 0 && pm) {
        const int p = (i - 1) + L.nx * (ly + G.L2 * (kk - 1));
        const float v = f3t_psi(G.bH[1][j], G.psiH[1][1][p], G.cH[1][j], ex_jp - ex_c);
        if (pm == 2) A.psiH_out[1][1][p] = v;
        h = __fmaf_rn(dt_mu0, v, h);
    }
    return h;
}

// The ADE of one dispersive component-cell: ade_update's arithmetic in the same order, with the
// pole state read again in the second loop instead of held in register arrays (which would take
// registers from the whole pass).  st: the cell's state at slot 0 (PD), V: the slot stride, P:
// poles per cell in the state.
__device__ __forceinline__ float f3t_ade(float e, float rot, int type, const MedR<float> *mp, float *st, long long V,
                                         int P)
{
    const MedR<float> &m = *mp;
    const float PD = st[0];
    if (type == CLS_DRUDE) {
        const float t = m.C1 * e + m.C3 * rot - m.C4 * PD;
        st[0] = m.A1 * PD + m.A2 * (t + e);
        return t;
    }
    const float eo = st[V];
    float t = m.C1 * e + m.C2 * eo + m.C3 * rot - m.C4 * PD;
    const int np = m.np;
#pragma unroll 1
    for (int p = 0; p < np; ++p) t = t - m.B1[p] * st[(2 + p) * V] - m.B2[p] * st[(2 + P + p) * V];
    st[0] = m.A1 * PD + m.A2 * (t + e);
#pragma unroll 1
    for (int p = 0; p < np; ++p) {
        const float pl = st[(2 + p) * V], plo = st[(2 + P + p) * V];
        st[(2 + P + p) * V] = pl;
        st[(2 + p) * V] = m.al[p] * pl + m.be[p] * plo + m.ga[p] * (t - eo);
    }
    st[V] = e;
    return t;
}

// E of one component inside the media box: plain classes, or the ADE of a dispersive class
__device__ __forceinline__ float f3t_media(float e, float rot, int c, int b, const GridArgs<float> &G)
{
    const ClsR<float> cl = G.cls[G.mat[c][b]];
    if (cl.type == CLS_PLAIN) return e + cl.coef * rot;
    return f3t_ade(e, rot, cl.type, G.med + cl.medium, G.ade + (long long)c * (2 + 2 * G.P) * G.bbV + b, G.bbV, G.P);
}

template <int TY> constexpr int f3t_min_blocks() { return TY == 8 ? 3 : 2; }

// One block's work: tile (bx, by) of 32 x TY columns over plane chunk bz of one grid.  maps: the
// in set's tensor maps (kernel parameter or global memory); nblk: the blocks of this grid's pass
// (the last of them to finish advances the grid's device-loop step counter); smem: the dynamic
// shared memory (F3tShape<TY>::SMEM bytes, 1024-byte aligned).
template <int TY>
__device__ __forceinline__ void f3t_tile(const CUtensorMap *maps, const Fused3Args &A, const GridArgs<float> &G,
                                         int bx, int by, int bz, int kch, unsigned nblk, int *err,
                                         unsigned char *f3_smem)
{
    using S = F3tShape<TY>;
    constexpr int NC = TY + 1;                 // warps that read the ring: compute + halo
    float *ring = reinterpret_cast<float *>(f3_smem);
    float *hn = reinterpret_cast<float *>(f3_smem + F3T_D * S::SLOTB);   // [2][3][TY+1][33]
    uint64_t *full = reinterpret_cast<uint64_t *>(f3_smem + F3T_D * S::SLOTB + 2 * 3 * S::HNF * 4);
    uint64_t *empty = full + F3T_D;
    const Lay &L = G.L;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i0 = 1 + bx * 32, j0 = 1 + by * TY;
    const int k0 = 1 + bz * kch, k1 = min(L.nz, k0 + kch - 1);
    const bool perz = G.per[2] != 0;
    // staged planes pa .. k1+1; pa = k0-1 when the new H of plane k0-1 is needed (k0 > 1, or the
    // periodic image of plane 0), else k0 (plane 0 is the PEC ghost: new H = 0)
    const int pa = (k0 > 1 || perz) ? k0 - 1 : k0;
    const int nq = k1 + 2 - pa;
    if (threadIdx.x == 0) {
        for (int s = 0; s < F3T_D; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], NC);
        }
        mbar_fence_init();
    }
    __syncthreads();

    if (warp == TY + 1) {
        // ---- copy warp: lane 0 stages plane pa + q into slot q % D
        if (lane != 0) return;
        int q = 0;
        bool ok = true;
        for (; q < nq; ++q) {
            const int s = q % F3T_D;
            if (q >= F3T_D && !mbar_wait_bounded(&empty[s], (uint32_t)(((q / F3T_D) - 1) & 1), F3T_WAIT_CYCLES)) {
                ok = false;
                break;
            }
            const int p = pa + q;
            const int z = (perz && p == 0) ? L.nz : ((perz && p == L.nz + 1) ? 1 : p);
            mbar_arrive_expect_tx(&full[s], 6u * S::BOXF * 4u);
            float *dst = ring + (size_t)s * (S::SLOTB / 4);
#pragma unroll
            for (int c = 0; c < 6; ++c)
                tma_load_3d(dst + c * (S::BOXB / 4), &maps[c], 32 * bx, j0 - 1, z, &full[s]);
        }
        if (!ok) {
            atomicOr(err, 1);
            for (int p = max(0, q - F3T_D); p < q; ++p)
                mbar_wait_bounded(&full[p % F3T_D], (uint32_t)((p / F3T_D) & 1), F3T_WAIT_CYCLES);
        }
        return;
    }

    // ---- compute warps (warp < TY: row j0 + warp) and the halo warp (warp == TY)
    const bool cw = warp < TY;
    const float dt_mu0 = G.dt_mu0, dt_eps0 = G.dt_eps0;
    // this thread's cell: compute warps own (i0 + lane, j0 + warp); the halo warp takes the row
    // halo cell (i0 + lane, j0 - 1) and, for lane < TY, the column halo cell (i0 - 1, j0 + lane)
    const int i = i0 + lane;
    const int j = cw ? j0 + warp : j0 - 1;
    const bool own = cw && i <= L.nx && j <= L.ny;
    const int ic = min(i, L.nx), jc = max(1, min(j, L.ny));
    const float dhx = G.den_h[0][ic], dhy = G.den_h[1][jc], dex = G.den_e[0][ic], dey = G.den_e[1][jc];
    const int lhx = G.lH[0][ic], lhy = G.lH[1][jc], lex = G.lE[0][ic], ley = G.lE[1][jc];
    // halo cells: row (i, j0 - 1) valid when j0 > 1 and i <= nx; column (i0 - 1, jh) when i0 > 1,
    // lane < TY and jh <= ny (a non-periodic index 0 is the PEC ghost: new H = 0)
    const bool row_h = !cw && j0 > 1 && i <= L.nx;
    const bool col_h = !cw && i0 > 1 && lane < TY && j0 + lane <= L.ny;
    const bool bb_ij = own && i >= G.bb0[0] && i <= G.bb1[0] && j >= G.bb0[1] && j <= G.bb1[1];
    const int col = (int)L.off + i + L.px * j;   // element offsets < 2^31 (checked by the host)
    const int cc = lane + 4;                   // staged column of i; row of j: warp + 1 (row halo: 0)
    const int rr = cw ? warp + 1 : 0;

    bool fail = false;
    float hxm = 0.f, hym = 0.f;                // new Hx, Hy of this cell at plane k - 1
    if (pa < k0) {
        // new H of plane pa = k0 - 1 (or the image of plane 0) for the owned cells, no writes
        fail |= !mbar_wait_bounded(&full[0], 0u, F3T_WAIT_CYCLES);
        fail |= !mbar_wait_bounded(&full[1], 0u, F3T_WAIT_CYCLES);
        if (cw) {
            const int kk = (pa == 0) ? L.nz : pa;
            const float *B0 = ring, *B1 = ring + S::SLOTB / 4;
            const int o = rr * F3T_BX + cc;
            const float ex_c = B0[o], ey_c = B0[S::BOXB / 4 + o], ez_c = B0[2 * (S::BOXB / 4) + o];
            const float ez_jp = B0[2 * (S::BOXB / 4) + o + F3T_BX], ez_ip = B0[2 * (S::BOXB / 4) + o + 1];
            const float ex_kp = B1[o], ey_kp = B1[S::BOXB / 4 + o];
            const float dhz = G.den_h[2][kk];
            const int lhz = G.lH[2][kk];
            hxm = f3t_hx(B0[3 * (S::BOXB / 4) + o], ez_c, ez_jp, ey_c, ey_kp, dhy, dhz, dt_mu0, lhy, lhz, G, A, ic, jc,
                         kk, own ? 1 : 0);
            hym = f3t_hy(B0[4 * (S::BOXB / 4) + o], ez_c, ez_ip, ex_c, ex_kp, dhx, dhz, dt_mu0, lhx, lhz, G, A, ic, jc,
                         kk, own ? 1 : 0);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[0]);
    }

    for (int k = k0; k <= k1; ++k) {
        const int q = k - pa, sc = q % F3T_D, sn = (q + 1) % F3T_D;
        fail |= !mbar_wait_bounded(&full[sc], (uint32_t)((q / F3T_D) & 1), F3T_WAIT_CYCLES);
        fail |= !mbar_wait_bounded(&full[sn], (uint32_t)(((q + 1) / F3T_D) & 1), F3T_WAIT_CYCLES);
        const float *Bc = ring + (size_t)sc * (S::SLOTB / 4);
        const float *Bn = ring + (size_t)sn * (S::SLOTB / 4);
        constexpr int CB = S::BOXB / 4;
        const float *Exc = Bc, *Eyc = Bc + CB, *Ezc = Bc + 2 * CB, *Hxc = Bc + 3 * CB, *Hyc = Bc + 4 * CB,
                    *Hzc = Bc + 5 * CB;
        const float dhz = G.den_h[2][k], dez = G.den_e[2][k];
        const int lhz = G.lH[2][k], lez = G.lE[2][k];
        float *hp = hn + (k & 1) * 3 * S::HNF;   // [Hx, Hy, Hz][TY+1][33]
        if (cw) {
            // new H of the own cell: into the tile in shared memory and out to HBM (nothing of it
            // stays in registers across the barrier; the E half reads it back)
            const int o = rr * F3T_BX + cc;
            const float ex_c = Exc[o], ey_c = Eyc[o], ez_c = Ezc[o];
            const float ez_jp = Ezc[o + F3T_BX], ez_ip = Ezc[o + 1];
            const float ey_ip = Eyc[o + 1], ex_jp = Exc[o + F3T_BX];
            const float ex_kp = Bn[o], ey_kp = Bn[CB + o];
            const float hx = f3t_hx(Hxc[o], ez_c, ez_jp, ey_c, ey_kp, dhy, dhz, dt_mu0, lhy, lhz, G, A, ic, jc, k,
                                    own ? 2 : 0);
            const float hy = f3t_hy(Hyc[o], ez_c, ez_ip, ex_c, ex_kp, dhx, dhz, dt_mu0, lhx, lhz, G, A, ic, jc, k,
                                    own ? 2 : 0);
            const float hz = f3t_hz(Hzc[o], ey_c, ey_ip, ex_c, ex_jp, dhx, dhy, dt_mu0, lhx, lhy, G, A, ic, jc, k,
                                    own ? 2 : 0);
            const int h = rr * 33 + lane + 1;
            hp[h] = hx;
            hp[S::HNF + h] = hy;
            hp[2 * S::HNF + h] = hz;
            if (own) {
                const int idx = col + (int)L.pz * k;
                __stcs(A.out.f[3] + idx, hx);
                __stcs(A.out.f[4] + idx, hy);
                __stcs(A.out.f[5] + idx, hz);
                if (perz && k == L.nz) {   // periodic ghost plane H(0) = H(nz) (mxll_3D_mod.f90:725-738)
                    A.out.f[3][idx - L.nz * (int)L.pz] = hx;
                    A.out.f[4][idx - L.nz * (int)L.pz] = hy;
                }
            }
        } else {
            // row halo (i, j0 - 1): Hz and Hx
            float rx = 0.f, rz = 0.f;
            if (row_h) {
                const int o = cc;                      // staged row 0
                const float e_x = Exc[o], e_y = Eyc[o], e_z = Ezc[o];
                rx = f3t_hx(Hxc[o], e_z, Ezc[o + F3T_BX], e_y, Bn[CB + o], dhy, dhz, dt_mu0, lhy, lhz, G, A, ic,
                            j0 - 1, k, 1);
                rz = f3t_hz(Hzc[o], e_y, Eyc[o + 1], e_x, Exc[o + F3T_BX], dhx, dhy, dt_mu0, lhx, lhy, G, A, ic,
                            j0 - 1, k, 1);
            }
            hp[lane + 1] = rx;
            hp[2 * S::HNF + lane + 1] = rz;
            // column halo (i0 - 1, jh): Hz and Hy
            if (lane < TY) {
                float cy = 0.f, cz = 0.f;
                if (col_h) {
                    const int ih = i0 - 1, jhc = j0 + lane;
                    const float dhx_h = G.den_h[0][ih], dhy_h = G.den_h[1][jhc];
                    const int lhx_h = G.lH[0][ih], lhy_h = G.lH[1][jhc];
                    const int o = (lane + 1) * F3T_BX + 3;
                    const float e_x = Exc[o], e_y = Eyc[o], e_z = Ezc[o];
                    cy = f3t_hy(Hyc[o], e_z, Ezc[o + 1], e_x, Bn[o], dhx_h, dhz, dt_mu0, lhx_h, lhz, G, A, ih, jhc, k, 1);
                    cz = f3t_hz(Hzc[o], e_y, Eyc[o + 1], e_x, Exc[o + F3T_BX], dhx_h, dhy_h, dt_mu0, lhx_h, lhy_h, G,
                                A, ih, jhc, k, 1);
                }
                hp[S::HNF + (lane + 1) * 33] = cy;
                hp[2 * S::HNF + (lane + 1) * 33] = cz;
            }
        }
        // the new-H tile is complete; every consumer warp learns whether any wait ran out
        if (bar_any(1, 32 * NC, fail)) {
            if (threadIdx.x == 0) atomicOr(err, 1);
            break;
        }
        if (cw) {
            const int idx = col + (int)L.pz * k;
            const int h = rr * 33 + lane + 1;
            const float hx = hp[h], hy = hp[S::HNF + h], hz = hp[2 * S::HNF + h];
            const int o = rr * F3T_BX + cc;
            const float ex_c = Exc[o], ey_c = Eyc[o], ez_c = Ezc[o];
            const float hz_im = hp[2 * S::HNF + h - 1], hy_im = hp[S::HNF + h - 1];
            const float hz_jm = hp[2 * S::HNF + h - 33], hx_jm = hp[h - 33];
            const float rx = (hz - hz_jm) * dey + (hym - hy) * dez;
            const float ry = (hz_im - hz) * dex + (hx - hxm) * dez;
            const float rz = (hy - hy_im) * dex + (hx_jm - hx) * dey;
            float ex = ex_c, ey = ey_c, ez = ez_c;
            if (G.pl_on && (G.pl_axis == 0 ? i : (G.pl_axis == 1 ? j : k)) == G.pl_index) {
                // the plane source of this step (source_interactions before the E update)
                const double a = sp_get(G.pl_amp);
                if (a != 0.0) {
                    const double add = __dmul_rn(G.pl_c_src, a);
                    if (G.pl_comp == 0) ex = (float)__dadd_rn((double)ex, add);
                    else if (G.pl_comp == 1) ey = (float)__dadd_rn((double)ey, add);
                    else ez = (float)__dadd_rn((double)ez, add);
                }
            }
            if (bb_ij && k >= G.bb0[2] && k <= G.bb1[2]) {
                const int b = (i - G.bb0[0]) + G.bbd[0] * ((j - G.bb0[1]) + G.bbd[1] * (k - G.bb0[2]));
                ex = f3t_media(ex, rx, 0, b, G);
                ey = f3t_media(ey, ry, 1, b, G);
                ez = f3t_media(ez, rz, 2, b, G);
            } else {
                ex = ex + dt_eps0 * rx;
                ey = ey + dt_eps0 * ry;
                ez = ez + dt_eps0 * rz;
            }
            if (own) {
                if (lex >= 0) {   // mxll_3D_mod.f90:817-849
                    const int p = lex + G.L2 * ((j - 1) + L.ny * (k - 1));
                    const float b = G.bE[0][i], c = G.cE[0][i];
                    const float v0 = b * G.psiE[0][0][p] + c * (hz_im - hz);
                    const float v1 = b * G.psiE[0][1][p] + c * (hy - hy_im);
                    G.psiE[0][0][p] = v0;
                    G.psiE[0][1][p] = v1;
                    ey = ey + dt_eps0 * v0;
                    ez = ez + dt_eps0 * v1;
                }
                if (ley >= 0) {   // :851-885
                    const int p = (i - 1) + L.nx * (ley + G.L2 * (k - 1));
                    const float b = G.bE[1][j], c = G.cE[1][j];
                    const float v0 = b * G.psiE[1][0][p] + c * (hz - hz_jm);
                    const float v1 = b * G.psiE[1][1][p] + c * (hx_jm - hx);
                    G.psiE[1][0][p] = v0;
                    G.psiE[1][1][p] = v1;
                    ex = ex + dt_eps0 * v0;
                    ez = ez + dt_eps0 * v1;
                }
                if (lez >= 0) {   // :887-921
                    const int p = (i - 1) + L.nx * ((j - 1) + L.ny * lez);
                    const float b = G.bE[2][k], c = G.cE[2][k];
                    const float v0 = b * G.psiE[2][0][p] + c * (hym - hy);
                    const float v1 = b * G.psiE[2][1][p] + c * (hx - hxm);
                    G.psiE[2][0][p] = v0;
                    G.psiE[2][1][p] = v1;
                    ex = ex + dt_eps0 * v0;
                    ey = ey + dt_eps0 * v1;
                }
                __stcs(A.out.f[0] + idx, ex);
                __stcs(A.out.f[1] + idx, ey);
                __stcs(A.out.f[2] + idx, ez);
            }
            hxm = hx;
            hym = hy;
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[sc]);   // plane k's slot is read
    }
    // device loop: the last block to finish advances the step counter, so every block of this
    // pass reads the step's scalars (the plane source amplitude) before the counter moves; the
    // host points those reads one table row ahead
    if (G.step_inc) {
        asm volatile("bar.sync 1, %0;" ::"r"(32 * NC) : "memory");
        if (threadIdx.x == 0) {
            __threadfence();
            if (atomicAdd((unsigned *)G.step_done, 1u) == nblk - 1) {
                *G.step_done = 0;
                *G.step_inc += 1;
                __threadfence();
            }
        }
    }
}

// The grid's arguments in shared memory, after the pass's own layout: read from there, the
// compiler does not hold the many pointers of the argument block in registers (which spilled).
template <int TY>
__device__ __forceinline__ void f3t_args_to_smem(const GridArgs<float> &G, const Fused3Args &A, unsigned char *smem)
{
    using S = F3tShape<TY>;
    const int *src = reinterpret_cast<const int *>(&G);
    int *dst = reinterpret_cast<int *>(smem + S::SMEM);
    for (int w = threadIdx.x; w < (int)(sizeof(GridArgs<float>) / 4); w += blockDim.x) dst[w] = src[w];
    src = reinterpret_cast<const int *>(&A);
    dst = reinterpret_cast<int *>(smem + S::SMEM + F3T_ARGB);
    for (int w = threadIdx.x; w < (int)(sizeof(Fused3Args) / 4); w += blockDim.x) dst[w] = src[w];
    __syncthreads();
}

template <int TY>
__global__ void __launch_bounds__(32 * (TY + 2), f3t_min_blocks<TY>())
    k_fused3_tma(const __grid_constant__ F3tMaps M, Fused3Args A, GridArgs<float> G, int kch, int *err)
{
    using S = F3tShape<TY>;
    extern __shared__ __align__(1024) unsigned char f3_smem[];
    f3t_args_to_smem<TY>(G, A, f3_smem);
    f3t_tile<TY>(M.m, *reinterpret_cast<const Fused3Args *>(f3_smem + S::SMEM + F3T_ARGB),
                 *reinterpret_cast<const GridArgs<float> *>(f3_smem + S::SMEM), (int)blockIdx.x, (int)blockIdx.y,
                 (int)blockIdx.z, kch, gridDim.x * gridDim.y * gridDim.z, err, f3_smem);
}

// ---- batched: the fused pass of several grids in one launch ----------------------------------
// Block b takes block b - item0 of the grid whose item range holds it (grids in the order of the
// table, largest first, so that the small grids' blocks fill the tail); the grid's arguments are
// copied into shared memory first.  Each grid computes exactly what its own k_fused3_tma does
// (same f3t_tile arithmetic; every tile shape gives the same bits).
template <int TY>
__global__ void __launch_bounds__(32 * (TY + 2), f3t_min_blocks<TY>())
    k_fused3_batch(const F3tBatchGrid *__restrict__ grids, int n, int *err)
{
    using S = F3tShape<TY>;
    extern __shared__ __align__(1024) unsigned char f3_smem[];
    const long long b = blockIdx.x;
    int lo = 0, hi = n - 1;                    // last grid with item0 <= b
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (grids[mid].item0 <= b) lo = mid;
        else hi = mid - 1;
    }
    const F3tBatchGrid &B = grids[lo];
    f3t_args_to_smem<TY>(B.G, B.A, f3_smem);
    const GridArgs<float> *sG = reinterpret_cast<const GridArgs<float> *>(f3_smem + S::SMEM);
    const Fused3Args *sA = reinterpret_cast<const Fused3Args *>(f3_smem + S::SMEM + F3T_ARGB);
    const long long t = b - B.item0;
    const int bx = (int)(t % B.tx), by = (int)((t / B.tx) % B.ty), bz = (int)(t / ((long long)B.tx * B.ty));
    f3t_tile<TY>(B.m, *sA, *sG, bx, by, bz, B.kch, (unsigned)((long long)B.tx * B.ty * B.tz), err, f3_smem);
}

}  // namespace omx
