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
constexpr long long F3T_WAIT_CYCLES = 2000000000LL;   // about one second at the SM clock
constexpr int F3T_PF = 2;     // planes ahead whose CPML psi and media words are prefetched into L1

// bytes reserved for the copy of a grid's GridArgs in the kernels' shared memory
constexpr int F3T_ARGB = (int)((sizeof(GridArgs<float>) + 15) / 16 * 16);

// Shared memory of a block, for a ring of nd plane slots: the copies of the grid's arguments
// (GridArgs, Fused3Args), the ring (1024-byte aligned), the new-H tiles, the per-plane z
// coefficients (2 float4 a plane) and the 2 nd mbarriers.  TY tile rows, RPT rows per compute
// thread (1 for 8 rows, 2 for 16): TY / RPT compute warps, a halo warp, a copy warp.
template <int TY> struct F3tShape {
    static constexpr int RPT = TY / 8;
    static constexpr int NCW = TY / RPT;                       // compute warps
    static constexpr int BY = TY + 2;                          // staged rows j0-1 .. j0+TY
    static constexpr int BOXF = F3T_BX * BY;                   // floats per staged box
    static constexpr int BOXB = (BOXF * 4 + 127) / 128 * 128;  // bytes per box slot (128-byte aligned)
    static constexpr int SLOTB = 6 * BOXB;                     // one plane: Ex, Ey, Ez, Hx, Hy, Hz
    static constexpr int HNF = (TY + 1) * 33;                  // new-H tile incl. column i0-1 and row j0-1
    static constexpr int ARGS = F3T_ARGB + (int)((sizeof(Fused3Args) + 15) / 16 * 16);
    static constexpr int RING = (ARGS + 1023) / 1024 * 1024;
    static constexpr int THREADS = 32 * (NCW + 2);
    __host__ __device__ static constexpr int hn_off(int nd) { return RING + nd * SLOTB; }
    __host__ __device__ static constexpr int z_off(int nd) { return (hn_off(nd) + 2 * 3 * HNF * 4 + 15) / 16 * 16; }
    __host__ __device__ static constexpr int bar_off(int nd) { return z_off(nd) + (F3T_KMAX + 2) * 32; }
    __host__ __device__ static constexpr int smem(int nd) { return bar_off(nd) + 2 * nd * 8; }
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

// The in-set H psi of one cell at its psi indices px, py, pz (-1: the cell lies in no slab of that
// axis; all zero when on = false): every load is issued before any of them is used, so that a cell
// in two or three slabs waits for memory once.  The in set is read-only during the pass (the
// owner writes the out set).
struct F3tPsiH {
    float x0, x1, y0, y1, z0, z1;
};
__device__ __forceinline__ F3tPsiH f3t_load_psiH(const GridArgs<float> &G, int px, int py, int pz, bool on)
{
    F3tPsiH q{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (!on) return q;
    if (px >= 0) {
        q.x0 = __ldg(G.psiH[0][0] + px);
        q.x1 = __ldg(G.psiH[0][1] + px);
    }
    if (py >= 0) {
        q.y0 = __ldg(G.psiH[1][0] + py);
        q.y1 = __ldg(G.psiH[1][1] + py);
    }
    if (pz >= 0) {
        q.z0 = __ldg(G.psiH[2][0] + pz);
        q.z1 = __ldg(G.psiH[2][1] + pz);
    }
    return q;
}

// New H components (h3_tile's expressions, the CPML faces in the reference's order) from the
// staged neighbourhood and the cell's in-set psi (f3t_load_psiH) at psi indices px / py / pz (-1:
// no slab).  i, j, kk: the cell's indices for the CPML coefficients of the faces it uses.  pm: 0
// no psi (a cell past the grid edge, whose value nobody uses, or a plane of the lean form), 1
// psi read only (a halo cell, or the plane before the first), 2 the new psi written to the out
// set (the owner).
__device__ __forceinline__ float f3t_hx(float hx, float ez_c, float ez_jp, float ey_c, float ey_kp, float dhy,
                                        float dhz, float dt_mu0, const GridArgs<float> &G, const Fused3Args &A,
                                        int j, int kk, int pm, int py, int pz, float psy, float psz)
{
    float h = __fmaf_rn(dt_mu0, __fmaf_rn(ey_kp - ey_c, dhz, __fmul_rn(ez_c - ez_jp, dhy)), hx);
    if (py >= 0 && pm) {   // mxll_3D_mod.f90:622-657
        const float v = f3t_psi(__ldg(G.bH[1] + j), psy, __ldg(G.cH[1] + j), ez_c - ez_jp);
        if (pm == 2) A.psiH_out[1][0][py] = v;
        h = __fmaf_rn(dt_mu0, v, h);
    }
    if (pz >= 0 && pm) {   // :659-694
        const float v = f3t_psi(__ldg(G.bH[2] + kk), psz, __ldg(G.cH[2] + kk), ey_kp - ey_c);
        if (pm == 2) A.psiH_out[2][0][pz] = v;
        h = __fmaf_rn(dt_mu0, v, h);
    }
    return h;
}
__device__ __forceinline__ float f3t_hy(float hy, float ez_c, float ez_ip, float ex_c, float ex_kp, float dhx,
                                        float dhz, float dt_mu0, const GridArgs<float> &G, const Fused3Args &A,
                                        int i, int kk, int pm, int px, int pz, float psx, float psz)
{
    float h = __fmaf_rn(dt_mu0, __fmaf_rn(ex_c - ex_kp, dhz, __fmul_rn(ez_ip - ez_c, dhx)), hy);
    if (px >= 0 && pm) {   // mxll_3D_mod.f90:585-620
        const float v = f3t_psi(__ldg(G.bH[0] + i), psx, __ldg(G.cH[0] + i), ez_ip - ez_c);
        if (pm == 2) A.psiH_out[0][0][px] = v;
        h = __fmaf_rn(dt_mu0, v, h);
    }
    if (pz >= 0 && pm) {
        const float v = f3t_psi(__ldg(G.bH[2] + kk), psz, __ldg(G.cH[2] + kk), ex_c - ex_kp);
        if (pm == 2) A.psiH_out[2][1][pz] = v;
        h = __fmaf_rn(dt_mu0, v, h);
    }
    return h;
}
__device__ __forceinline__ float f3t_hz(float hz, float ey_c, float ey_ip, float ex_c, float ex_jp, float dhx,
                                        float dhy, float dt_mu0, const GridArgs<float> &G, const Fused3Args &A,
                                        int i, int j, int pm, int px, int py, float psx, float psy)
{
    float h = __fmaf_rn(dt_mu0, __fmaf_rn(ex_jp - ex_c, dhy, __fmul_rn(ey_c - ey_ip, dhx)), hz);
    if (px >= 0 && pm) {
        const float v = f3t_psi(__ldg(G.bH[0] + i), psx, __ldg(G.cH[0] + i), ey_c - ey_ip);
        if (pm == 2) A.psiH_out[0][1][px] = v;
        h = __fmaf_rn(dt_mu0, v, h);
    }
    if (py >= 0 && pm) {
        const float v = f3t_psi(__ldg(G.bH[1] + j), psy, __ldg(G.cH[1] + j), ex_jp - ex_c);
        if (pm == 2) A.psiH_out[1][1][py] = v;
        h = __fmaf_rn(dt_mu0, v, h);
    }
    return h;
}

// The ADE of one dispersive component-cell: ade_update's terms in the same order, each product
// added by an explicitly rounded FMA (so that no tile shape or code path contracts differently),
// with the pole state read again in the second loop instead of held in register arrays (which
// would take registers from the whole pass).  st: the cell's state at slot 0 (PD), V: the slot stride, P:
// poles per cell in the state.
__device__ __forceinline__ float f3t_ade(float e, float rot, int type, const MedR<float> *mp, float *st, long long V,
                                         int P)
{
    const MedR<float> &m = *mp;
    const float PD = st[0];
    if (type == CLS_DRUDE) {
        const float t = __fmaf_rn(-m.C4, PD, __fmaf_rn(m.C3, rot, __fmul_rn(m.C1, e)));
        st[0] = __fmaf_rn(m.A1, PD, __fmul_rn(m.A2, __fadd_rn(t, e)));
        return t;
    }
    const float eo = st[V];
    float t = __fmaf_rn(-m.C4, PD, __fmaf_rn(m.C3, rot, __fmaf_rn(m.C2, eo, __fmul_rn(m.C1, e))));
    const int np = m.np;
#pragma unroll 1
    for (int p = 0; p < np; ++p)
        t = __fmaf_rn(-m.B2[p], st[(2 + P + p) * V], __fmaf_rn(-m.B1[p], st[(2 + p) * V], t));
    st[0] = __fmaf_rn(m.A1, PD, __fmul_rn(m.A2, __fadd_rn(t, e)));
    const float dte = __fsub_rn(t, eo);
#pragma unroll 1
    for (int p = 0; p < np; ++p) {
        const float pl = st[(2 + p) * V], plo = st[(2 + P + p) * V];
        st[(2 + P + p) * V] = pl;
        st[(2 + p) * V] = __fmaf_rn(m.al[p], pl, __fmaf_rn(m.be[p], plo, __fmul_rn(m.ga[p], dte)));
    }
    st[V] = e;
    return t;
}

// E of one component inside the media box: plain classes, or the ADE of a dispersive class
__device__ __forceinline__ float f3t_media(float e, float rot, int c, int b, const GridArgs<float> &G)
{
    const ClsR<float> cl = G.cls[G.mat[c][b]];
    if (cl.type == CLS_PLAIN) return __fmaf_rn(cl.coef, rot, e);
    return f3t_ade(e, rot, cl.type, G.med + cl.medium, G.ade + (long long)c * (2 + 2 * G.P) * G.bbV + b, G.bbV, G.P);
}

// The curl of the new H at an owned cell (the E update's right-hand side per unit dt_eps0), every
// operation rounded explicitly so that every kernel and tile shape gives a cell the same bits.
// hxm, hym: new Hx, Hy of plane k-1; dhxk, dhyk: their plane differences (the z-face psi's input).
__device__ __forceinline__ void f3t_curl(float hx, float hy, float hz, float hz_im, float hy_im, float hz_jm,
                                         float hx_jm, float hxm, float hym, float dex, float dey, float dez, float &rx,
                                         float &ry, float &rz, float &dhxk, float &dhyk)
{
    dhyk = __fsub_rn(hym, hy);
    dhxk = __fsub_rn(hx, hxm);
    rx = __fmaf_rn(dhyk, dez, __fmul_rn(__fsub_rn(hz, hz_jm), dey));
    ry = __fmaf_rn(dhxk, dez, __fmul_rn(__fsub_rn(hz_im, hz), dex));
    rz = __fmaf_rn(__fsub_rn(hx_jm, hx), dey, __fmul_rn(__fsub_rn(hy, hy_im), dex));
}

// New E of an owned cell (i, j, k) in the general form, from its old E (in ex, ey, ez) and the
// curl of the new H: the plane source of the step, the media-box update (plain classes or the
// ADE) or the vacuum update, then the CPML E psi of the x, y and z faces in the reference's order
// (mxll_3D_mod.f90:740-921).  pe0, pe1, pe2: the cell's E psi indices (-1: no slab; in place: each
// word is read and written by this thread only, all of them requested first); bz, cz: the z
// face's coefficients of plane k; bbc: (i, j) lies in the media box's x-y extent.
__device__ __forceinline__ void f3t_e_general(float &ex, float &ey, float &ez, float rx, float ry, float rz, float dhxk,
                                              float dhyk, float hx, float hy, float hz, float hz_im, float hy_im,
                                              float hz_jm, float hx_jm, int i, int j, int k, int pe0, int pe1, int pe2,
                                              float bz, float cz, bool bbc, float dt_eps0, const GridArgs<float> &G)
{
    float qe[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (pe0 >= 0) {
        qe[0] = __ldg(G.psiE[0][0] + pe0);
        qe[1] = __ldg(G.psiE[0][1] + pe0);
    }
    if (pe1 >= 0) {
        qe[2] = __ldg(G.psiE[1][0] + pe1);
        qe[3] = __ldg(G.psiE[1][1] + pe1);
    }
    if (pe2 >= 0) {
        qe[4] = __ldg(G.psiE[2][0] + pe2);
        qe[5] = __ldg(G.psiE[2][1] + pe2);
    }
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
    if (bbc && k >= G.bb0[2] && k <= G.bb1[2]) {
        const int b = (i - G.bb0[0]) + G.bbd[0] * ((j - G.bb0[1]) + G.bbd[1] * (k - G.bb0[2]));
        ex = f3t_media(ex, rx, 0, b, G);
        ey = f3t_media(ey, ry, 1, b, G);
        ez = f3t_media(ez, rz, 2, b, G);
    } else {
        ex = __fmaf_rn(dt_eps0, rx, ex);
        ey = __fmaf_rn(dt_eps0, ry, ey);
        ez = __fmaf_rn(dt_eps0, rz, ez);
    }
    if (pe0 >= 0) {   // mxll_3D_mod.f90:817-849
        const float b = __ldg(G.bE[0] + i), c = __ldg(G.cE[0] + i);
        const float v0 = f3t_psi(b, qe[0], c, __fsub_rn(hz_im, hz));
        const float v1 = f3t_psi(b, qe[1], c, __fsub_rn(hy, hy_im));
        G.psiE[0][0][pe0] = v0;
        G.psiE[0][1][pe0] = v1;
        ey = __fmaf_rn(dt_eps0, v0, ey);
        ez = __fmaf_rn(dt_eps0, v1, ez);
    }
    if (pe1 >= 0) {   // :851-885
        const float b = __ldg(G.bE[1] + j), c = __ldg(G.cE[1] + j);
        const float v0 = f3t_psi(b, qe[2], c, __fsub_rn(hz, hz_jm));
        const float v1 = f3t_psi(b, qe[3], c, __fsub_rn(hx_jm, hx));
        G.psiE[1][0][pe1] = v0;
        G.psiE[1][1][pe1] = v1;
        ex = __fmaf_rn(dt_eps0, v0, ex);
        ez = __fmaf_rn(dt_eps0, v1, ez);
    }
    if (pe2 >= 0) {   // :887-921
        const float v0 = f3t_psi(bz, qe[4], cz, dhyk);
        const float v1 = f3t_psi(bz, qe[5], cz, dhxk);
        G.psiE[2][0][pe2] = v0;
        G.psiE[2][1][pe2] = v1;
        ex = __fmaf_rn(dt_eps0, v0, ex);
        ey = __fmaf_rn(dt_eps0, v1, ey);
    }
}

template <int TY> constexpr int f3t_min_blocks() { return 2; }

// the form a plane is computed in: lean (no CPML psi, media or plane source at the block's cells
// of the plane) or general
template <bool B> struct F3tForm {
    static constexpr bool value = B;
};

// prefetch the 128-byte line of p into L1 (the next plane's CPML and media words)
__device__ __forceinline__ void f3t_prefetch(const void *p)
{
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// How a launch chooses the form of each plane: per plane (F3T_MIXED, the batched pass) or every
// plane lean (F3T_LEAN_ONLY: the host gave this launch lean runs only; the general code is not
// compiled in, which keeps the lean form's registers to itself).
enum { F3T_MIXED = 0, F3T_LEAN_ONLY = 1 };

// One block's work: the tile of 32 x TY columns from (i0, j0) over planes k0 .. k1 of one grid
// (i0 = 1 mod 4: the staged box starts at i0 - 4 on a 16-byte boundary).  maps: the
// in set's tensor maps (kernel parameter or global memory); A, G: the grid's arguments (in
// shared memory); nblk: the blocks of this launch (the last of them to finish advances the
// grid's device-loop step counter, when G.step_inc is set); smem: the dynamic shared memory
// (1024-byte aligned).
template <int TY, int MODE>
__device__ __forceinline__ void f3t_tile(const CUtensorMap *maps, const Fused3Args &A, const GridArgs<float> &G,
                                         int i0, int j0, int k0, int k1, int nd, unsigned nblk, int *err,
                                         unsigned char *f3_smem)
{
    using S = F3tShape<TY>;
    constexpr int RPT = S::RPT, NCW = S::NCW;
    constexpr int NC = NCW + 1;                // warps that read the ring: compute + halo
    constexpr int CB = S::BOXB / 4;
    float *ring = reinterpret_cast<float *>(f3_smem + S::RING);           // [nd][6][box]
    float *hn = reinterpret_cast<float *>(f3_smem + S::hn_off(nd));      // [2][3][TY+1][33]
    float4 *zc = reinterpret_cast<float4 *>(f3_smem + S::z_off(nd));     // [plane - pa][2]
    uint64_t *full = reinterpret_cast<uint64_t *>(f3_smem + S::bar_off(nd));
    uint64_t *empty = full + nd;
    const Lay &L = G.L;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool perz = G.per[2] != 0;
    // staged planes pa .. k1+1; pa = k0-1 when the new H of plane k0-1 is needed (k0 > 1, or the
    // periodic image of plane 0), else k0 (plane 0 is the PEC ghost: new H = 0)
    const int pa = (k0 > 1 || perz) ? k0 - 1 : k0;
    const int nq = k1 + 2 - pa;
    if (threadIdx.x == 0) {
        for (int s = 0; s < nd; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], NC);
        }
        mbar_fence_init();
    }
    // per-plane z coefficients of the planes pa .. k1 (index of plane 0 of a periodic axis: nz):
    // (den_h, den_e, bH, cH) and (bE, cE, H psi layer, E psi layer)
    for (int t = threadIdx.x; t < nq - 1; t += blockDim.x) {
        const int p = pa + t, kk = p == 0 ? L.nz : p;
        const int lh = G.lH[2][kk], le = G.lE[2][kk];
        zc[2 * t] = make_float4(G.den_h[2][kk], G.den_e[2][kk], G.bH[2][kk], G.cH[2][kk]);
        zc[2 * t + 1] = make_float4(G.bE[2][kk], G.cE[2][kk], __int_as_float(lh), __int_as_float(le));
    }
    // does a CPML slab of x or y reach a cell this block updates (own or halo)?  Then every plane
    // takes the general form; else a plane without z CPML, media or plane source takes the lean one
    bool slab = false;
    if (threadIdx.x < 33) {
        const int ih = i0 - 1 + (int)threadIdx.x;
        if (ih >= 1 && ih <= L.nx) slab = G.lH[0][ih] >= 0 || G.lE[0][ih] >= 0;
    } else if (threadIdx.x < 34 + TY) {
        const int jh = j0 - 34 + (int)threadIdx.x;
        if (jh >= 1 && jh <= L.ny) slab = G.lH[1][jh] >= 0 || G.lE[1][jh] >= 0;
    }
    const bool xy_slab = __syncthreads_or(slab) != 0;

    if (warp == NCW + 1) {
        // ---- copy warp: lane 0 stages plane pa + q into slot q % D
        if (lane != 0) return;
        int q = 0, s = 0, round = 0;           // plane q goes to slot s in its round-th use
        bool ok = true;
        for (; q < nq; ++q) {
            if (round > 0 && !mbar_wait_bounded(&empty[s], (uint32_t)((round - 1) & 1), F3T_WAIT_CYCLES)) {
                ok = false;
                break;
            }
            const int p = pa + q;
            const int z = (perz && p == 0) ? L.nz : ((perz && p == L.nz + 1) ? 1 : p);
            mbar_arrive_expect_tx(&full[s], 6u * S::BOXF * 4u);
            float *dst = ring + (size_t)s * (S::SLOTB / 4);
#pragma unroll
            for (int c = 0; c < 6; ++c)
                tma_load_3d(dst + c * CB, &maps[c], i0 - 1, j0 - 1, z, &full[s]);
            if (++s == nd) {
                s = 0;
                ++round;
            }
        }
        if (!ok) {
            atomicOr(err, 1);
            for (int p = max(0, q - nd); p < q; ++p)
                mbar_wait_bounded(&full[p % nd], (uint32_t)((p / nd) & 1), F3T_WAIT_CYCLES);
        }
        return;
    }

    // ---- compute warps (warp < NCW: rows j0 + RPT warp + r) and the halo warp (warp == NCW)
    const bool cw = warp < NCW;
    const float dt_mu0 = G.dt_mu0, dt_eps0 = G.dt_eps0;
    const int i = i0 + lane;
    const int ic = min(i, L.nx);
    const float dhx = G.den_h[0][ic], dex = G.den_e[0][ic];
    const int cc = lane + 4;                   // staged column of i
    // CPML psi offsets of the planes: x and y faces grow by one plane of their array per k, the z
    // face holds sZ words per layer
    const int sX = G.L2 * L.ny, sY = L.nx * G.L2, sZ = L.nx * L.ny;
    // compute warps: cells (i, j_r), j_r = j0 + RPT warp + r, staged row rr_r = j_r - j0 + 1.  The
    // halo warp: the row halo cell (i, j0 - 1) as its row 0 and, for lane < TY, the column halo
    // cell (i0 - 1, j0 + lane) (a non-periodic index 0 is the PEC ghost: new H = 0).  Per row, the
    // psi index of each face at plane 1 (x, y) or layer 0 (z); -1 where the cell is in no slab.
    const int jb = cw ? j0 + RPT * warp : j0 - 1;
    const int lhx = G.lH[0][ic], lex = G.lE[0][ic];
    float dhy[RPT], dey[RPT];
    int bxH[RPT], bxE[RPT], byH[RPT], byE[RPT], bz0[RPT];
    bool own[RPT], bbc[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
        const int j = jb + r, jc = max(1, min(j, L.ny));
        dhy[r] = G.den_h[1][jc];
        dey[r] = G.den_e[1][jc];
        const int lhy = G.lH[1][jc], ley = G.lE[1][jc];
        bxH[r] = lhx >= 0 ? lhx + G.L2 * (jc - 1) : -1;
        bxE[r] = lex >= 0 ? lex + G.L2 * (jc - 1) : -1;
        byH[r] = lhy >= 0 ? (ic - 1) + L.nx * lhy : -1;
        byE[r] = ley >= 0 ? (ic - 1) + L.nx * ley : -1;
        bz0[r] = (ic - 1) + L.nx * (jc - 1);
        own[r] = cw && i <= L.nx && j <= L.ny;
        bbc[r] = own[r] && i >= G.bb0[0] && i <= G.bb1[0] && j >= G.bb0[1] && j <= G.bb1[1];
    }
    const bool row_h = !cw && j0 > 1 && i <= L.nx;
    const bool col_h = !cw && i0 > 1 && lane < TY && j0 + lane <= L.ny;
    // the column halo cell (i0 - 1, jhc) of this lane and its psi bases
    const int ih = i0 - 1, jhc = min(j0 + lane, L.ny);
    int cxH = -1, cyH = -1, cz0 = 0;
    if (col_h) {
        const int lx = G.lH[0][ih], ly = G.lH[1][jhc];
        cxH = lx >= 0 ? lx + G.L2 * (jhc - 1) : -1;
        cyH = ly >= 0 ? (ih - 1) + L.nx * ly : -1;
        cz0 = (ih - 1) + L.nx * (jhc - 1);
    }
    const int col0 = (int)L.off + i + L.px * jb;   // element offsets < 2^31 (checked by the host)
    const int rr0 = cw ? RPT * warp + 1 : 0;
    // psi indices of a face at plane kk: x / y from a plane-1 base, z from the layer lz
    auto at_x = [&](int b, int kk) { return b >= 0 ? b + sX * (kk - 1) : -1; };
    auto at_y = [&](int b, int kk) { return b >= 0 ? b + sY * (kk - 1) : -1; };
    auto at_z = [&](int b, int lz) { return lz >= 0 ? b + sZ * lz : -1; };

    bool fail = false;
    float hxm[RPT], hym[RPT];                  // new Hx, Hy of the own cells at plane k - 1
#pragma unroll
    for (int r = 0; r < RPT; ++r) hxm[r] = hym[r] = 0.f;
    if (pa < k0) {
        // new H of plane pa = k0 - 1 (or the image of plane 0) for the owned cells, no writes
        fail |= !mbar_wait_bounded(&full[0], 0u, F3T_WAIT_CYCLES);
        fail |= !mbar_wait_bounded(&full[1], 0u, F3T_WAIT_CYCLES);
        if (cw) {
            const int kk = (pa == 0) ? L.nz : pa;
            const float *B0 = ring, *B1 = ring + S::SLOTB / 4;
            const float4 z0 = zc[0], z1 = zc[1];
            const int lhz = __float_as_int(z1.z);
#pragma unroll
            for (int r = 0; r < RPT; ++r) {
                const int o = (rr0 + r) * F3T_BX + cc;
                const float ex_c = B0[o], ey_c = B0[CB + o], ez_c = B0[2 * CB + o];
                const float ez_jp = B0[2 * CB + o + F3T_BX], ez_ip = B0[2 * CB + o + 1];
                const float ex_kp = B1[o], ey_kp = B1[CB + o];
                const int jc = max(1, min(jb + r, L.ny));
                const int px = at_x(bxH[r], kk), py = at_y(byH[r], kk), pz = at_z(bz0[r], lhz);
                const F3tPsiH q = f3t_load_psiH(G, px, py, pz, own[r]);
                hxm[r] = f3t_hx(B0[3 * CB + o], ez_c, ez_jp, ey_c, ey_kp, dhy[r], z0.x, dt_mu0, G, A, jc, kk,
                                own[r] ? 1 : 0, py, pz, q.y0, q.z0);
                hym[r] = f3t_hy(B0[4 * CB + o], ez_c, ez_ip, ex_c, ex_kp, dhx, z0.x, dt_mu0, G, A, ic, kk,
                                own[r] ? 1 : 0, px, pz, q.x0, q.z1);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[0]);
    } else {
        fail |= !mbar_wait_bounded(&full[0], 0u, F3T_WAIT_CYCLES);
    }

    // Planes that need none of the CPML psi, the media box or the plane source take the lean
    // form (the same expressions with those branches left out): no x / y slab at the block's
    // cells, no z slab at the plane, no media-box cell in the tile's part of the plane, no
    // source plane through the tile.
    const bool mb_xy = G.bb1[0] >= G.bb0[0] && G.bb1[1] >= G.bb0[1] && G.bb1[2] >= G.bb0[2] &&
                       G.bb0[0] <= i0 + 31 && G.bb1[0] >= i0 && G.bb0[1] <= j0 + TY - 1 && G.bb1[1] >= j0;
    const int mbk0 = mb_xy ? G.bb0[2] : 1, mbk1 = mb_xy ? G.bb1[2] : 0;
    const bool pl_xy = G.pl_on && ((G.pl_axis == 0 && G.pl_index >= i0 && G.pl_index <= i0 + 31) ||
                                   (G.pl_axis == 1 && G.pl_index >= j0 && G.pl_index <= j0 + TY - 1));
    const int plk = (G.pl_on && G.pl_axis == 2) ? G.pl_index : -1;
    auto lean_at = [&](int k, float4 z1) {
        return !xy_slab && !pl_xy && __float_as_int(z1.z) < 0 && __float_as_int(z1.w) < 0 && k != plk &&
               (k < mbk0 || k > mbk1);
    };

    // One plane: new H of the tile (+ halo) into shared memory and HBM, the barrier, then new E.
    // Returns true when a wait ran out somewhere in the block (every consumer warp then leaves).
    auto plane = [&](auto form, int k, int sc, int sn, float4 z0, float4 z1) -> bool {
        constexpr bool LEAN = decltype(form)::value;
        const float *Bc = ring + (size_t)sc * (S::SLOTB / 4);
        const float *Bn = ring + (size_t)sn * (S::SLOTB / 4);
        const float *Exc = Bc, *Eyc = Bc + CB, *Ezc = Bc + 2 * CB, *Hxc = Bc + 3 * CB, *Hyc = Bc + 4 * CB,
                    *Hzc = Bc + 5 * CB;
        const float dhz = z0.x;
        const int lhz = __float_as_int(z1.z);
        float *hp = hn + (k & 1) * 3 * S::HNF;   // [Hx, Hy, Hz][TY+1][33]
        float eo[RPT][3];                        // lean form: old E of the own cells across the barrier
        if (cw) {
            // new H of the own cells: into the tile in shared memory and out to HBM; every row's
            // psi is requested before any is used
            int px[RPT], py[RPT], pz[RPT];
            F3tPsiH q[RPT];
#pragma unroll
            for (int r = 0; r < RPT; ++r) {
                px[r] = LEAN ? -1 : at_x(bxH[r], k);
                py[r] = LEAN ? -1 : at_y(byH[r], k);
                pz[r] = LEAN ? -1 : at_z(bz0[r], lhz);
                q[r] = f3t_load_psiH(G, px[r], py[r], pz[r], !LEAN && own[r]);
            }
#pragma unroll
            for (int r = 0; r < RPT; ++r) {
                const int o = (rr0 + r) * F3T_BX + cc;
                const int jc = max(1, min(jb + r, L.ny));
                const float ex_c = Exc[o], ey_c = Eyc[o], ez_c = Ezc[o];
                const float ez_jp = Ezc[o + F3T_BX], ez_ip = Ezc[o + 1];
                const float ey_ip = Eyc[o + 1], ex_jp = Exc[o + F3T_BX];
                const float ex_kp = Bn[o], ey_kp = Bn[CB + o];
                if constexpr (LEAN) {
                    eo[r][0] = ex_c;
                    eo[r][1] = ey_c;
                    eo[r][2] = ez_c;
                }
                const int pm = (LEAN || !own[r]) ? 0 : 2;
                const float hx = f3t_hx(Hxc[o], ez_c, ez_jp, ey_c, ey_kp, dhy[r], dhz, dt_mu0, G, A, jc, k, pm, py[r],
                                        pz[r], q[r].y0, q[r].z0);
                const float hy = f3t_hy(Hyc[o], ez_c, ez_ip, ex_c, ex_kp, dhx, dhz, dt_mu0, G, A, ic, k, pm, px[r],
                                        pz[r], q[r].x0, q[r].z1);
                const float hz = f3t_hz(Hzc[o], ey_c, ey_ip, ex_c, ex_jp, dhx, dhy[r], dt_mu0, G, A, ic, jc, pm,
                                        px[r], py[r], q[r].x1, q[r].y1);
                const int h = (rr0 + r) * 33 + lane + 1;
                hp[h] = hx;
                hp[S::HNF + h] = hy;
                hp[2 * S::HNF + h] = hz;
                if (own[r]) {
                    const int idx = col0 + L.px * r + (int)L.pz * k;
                    __stcs(A.out.f[3] + idx, hx);
                    __stcs(A.out.f[4] + idx, hy);
                    __stcs(A.out.f[5] + idx, hz);
                    if (perz && k == L.nz) {   // periodic ghost plane H(0) = H(nz) (mxll_3D_mod.f90:725-738)
                        A.out.f[3][idx - L.nz * (int)L.pz] = hx;
                        A.out.f[4][idx - L.nz * (int)L.pz] = hy;
                    }
                }
            }
        } else {
            // row halo (i, j0 - 1): Hz and Hx; column halo (i0 - 1, j0 + lane): Hz and Hy (the psi of
            // both requested first)
            const int rxp = LEAN ? -1 : at_x(bxH[0], k), ryp = LEAN ? -1 : at_y(byH[0], k);
            const int rzp = LEAN ? -1 : at_z(bz0[0], lhz);
            const int cxp = LEAN ? -1 : at_x(cxH, k), cyp = LEAN ? -1 : at_y(cyH, k);
            const int czp = LEAN ? -1 : at_z(cz0, lhz);
            const F3tPsiH qr = f3t_load_psiH(G, rxp, ryp, rzp, !LEAN && row_h);
            const F3tPsiH qc = f3t_load_psiH(G, cxp, cyp, czp, !LEAN && col_h);
            float rx = 0.f, rz = 0.f;
            if (row_h) {
                const int o = cc;                      // staged row 0
                const float e_x = Exc[o], e_y = Eyc[o], e_z = Ezc[o];
                rx = f3t_hx(Hxc[o], e_z, Ezc[o + F3T_BX], e_y, Bn[CB + o], dhy[0], dhz, dt_mu0, G, A, j0 - 1, k,
                            LEAN ? 0 : 1, ryp, rzp, qr.y0, qr.z0);
                rz = f3t_hz(Hzc[o], e_y, Eyc[o + 1], e_x, Exc[o + F3T_BX], dhx, dhy[0], dt_mu0, G, A, ic, j0 - 1,
                            LEAN ? 0 : 1, rxp, ryp, qr.x1, qr.y1);
            }
            hp[lane + 1] = rx;
            hp[2 * S::HNF + lane + 1] = rz;
            if (lane < TY) {
                float cy = 0.f, cz = 0.f;
                if (col_h) {
                    const float dhx_h = G.den_h[0][ih], dhy_h = G.den_h[1][jhc];
                    const int o = (lane + 1) * F3T_BX + 3;
                    const float e_x = Exc[o], e_y = Eyc[o], e_z = Ezc[o];
                    cy = f3t_hy(Hyc[o], e_z, Ezc[o + 1], e_x, Bn[o], dhx_h, dhz, dt_mu0, G, A, ih, k, LEAN ? 0 : 1,
                                cxp, czp, qc.x0, qc.z1);
                    cz = f3t_hz(Hzc[o], e_y, Eyc[o + 1], e_x, Exc[o + F3T_BX], dhx_h, dhy_h, dt_mu0, G, A, ih, jhc,
                                LEAN ? 0 : 1, cxp, cyp, qc.x1, qc.y1);
                }
                hp[S::HNF + (lane + 1) * 33] = cy;
                hp[2 * S::HNF + (lane + 1) * 33] = cz;
            }
        }
        // the new-H tile is complete; every consumer warp learns whether any wait ran out
        if (bar_any(1, 32 * NC, fail)) return true;
        if (cw) {
            const float dez = z0.y;
            const int lez = __float_as_int(z1.w);
#pragma unroll
            for (int r = 0; r < RPT; ++r) {
                const int h = (rr0 + r) * 33 + lane + 1;
                const float hx = hp[h], hy = hp[S::HNF + h], hz = hp[2 * S::HNF + h];
                const float hz_im = hp[2 * S::HNF + h - 1], hy_im = hp[S::HNF + h - 1];
                const float hz_jm = hp[2 * S::HNF + h - 33], hx_jm = hp[h - 33];
                float rx, ry, rz, dhxk, dhyk;
                f3t_curl(hx, hy, hz, hz_im, hy_im, hz_jm, hx_jm, hxm[r], hym[r], dex, dey[r], dez, rx, ry, rz, dhxk,
                         dhyk);
                hxm[r] = hx;
                hym[r] = hy;
                if (!own[r]) continue;
                float ex, ey, ez;
                if constexpr (LEAN) {
                    ex = __fmaf_rn(dt_eps0, rx, eo[r][0]);
                    ey = __fmaf_rn(dt_eps0, ry, eo[r][1]);
                    ez = __fmaf_rn(dt_eps0, rz, eo[r][2]);
                } else {
                    const int o = (rr0 + r) * F3T_BX + cc;
                    ex = Exc[o];
                    ey = Eyc[o];
                    ez = Ezc[o];
                    f3t_e_general(ex, ey, ez, rx, ry, rz, dhxk, dhyk, hx, hy, hz, hz_im, hy_im, hz_jm, hx_jm, i, jb + r, k,
                                  at_x(bxE[r], k), at_y(byE[r], k), at_z(bz0[r], lez), z1.x, z1.y, bbc[r], dt_eps0, G);
                }
                const int idx = col0 + L.px * r + (int)L.pz * k;
                __stcs(A.out.f[0] + idx, ex);
                __stcs(A.out.f[1] + idx, ey);
                __stcs(A.out.f[2] + idx, ez);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[sc]);   // plane k's slot is read
        return false;
    };

    // slot and round of plane k (kept as counters: the ring depth is a launch parameter)
    int sc = k0 - pa, rc = 0;
    for (int k = k0; k <= k1; ++k) {
        const int q = k - pa;
        const int sn = sc + 1 == nd ? 0 : sc + 1, rn = sc + 1 == nd ? rc + 1 : rc;
        const float4 z0 = zc[2 * q], z1 = zc[2 * q + 1];
        // the words of plane kn = k + F3T_PF that come from HBM outside the staging (CPML psi,
        // media bytes) are pulled into L1 now, so that their loads there do not stall the block
        const int kn = k + F3T_PF;
        if (MODE != F3T_LEAN_ONLY && kn <= k1) {
            const float4 zn = zc[2 * (q + F3T_PF) + 1];
            if (!lean_at(kn, zn)) {
                const int lhzn = __float_as_int(zn.z), lezn = __float_as_int(zn.w);
                if (cw) {
#pragma unroll
                    for (int r = 0; r < RPT; ++r) {
                        if (!own[r]) continue;
                        const int pxh = at_x(bxH[r], kn), pxe = at_x(bxE[r], kn);
                        const int pyh = at_y(byH[r], kn), pye = at_y(byE[r], kn);
                        const int pzh = at_z(bz0[r], lhzn), pze = at_z(bz0[r], lezn);
                        if (pxh >= 0) {
                            f3t_prefetch(G.psiH[0][0] + pxh);
                            f3t_prefetch(G.psiH[0][1] + pxh);
                        }
                        if (pxe >= 0) {
                            f3t_prefetch(G.psiE[0][0] + pxe);
                            f3t_prefetch(G.psiE[0][1] + pxe);
                        }
                        if (pyh >= 0) {
                            f3t_prefetch(G.psiH[1][0] + pyh);
                            f3t_prefetch(G.psiH[1][1] + pyh);
                        }
                        if (pye >= 0) {
                            f3t_prefetch(G.psiE[1][0] + pye);
                            f3t_prefetch(G.psiE[1][1] + pye);
                        }
                        if (pzh >= 0) {
                            f3t_prefetch(G.psiH[2][0] + pzh);
                            f3t_prefetch(G.psiH[2][1] + pzh);
                        }
                        if (pze >= 0) {
                            f3t_prefetch(G.psiE[2][0] + pze);
                            f3t_prefetch(G.psiE[2][1] + pze);
                        }
                        const int j = jb + r;
                        if (bbc[r] && kn >= G.bb0[2] && kn <= G.bb1[2]) {
                            const int b = (i - G.bb0[0]) + G.bbd[0] * ((j - G.bb0[1]) + G.bbd[1] * (kn - G.bb0[2]));
                            f3t_prefetch(G.mat[0] + b);
                            f3t_prefetch(G.mat[1] + b);
                            f3t_prefetch(G.mat[2] + b);
                        }
                    }
                } else {
                    // the halo cells' in-set H psi (their loads would otherwise hold every
                    // compute warp at the plane's barrier for a trip to memory)
                    if (row_h) {
                        const int px = at_x(bxH[0], kn), py = at_y(byH[0], kn), pz = at_z(bz0[0], lhzn);
                        if (px >= 0) f3t_prefetch(G.psiH[0][1] + px);
                        if (py >= 0) {
                            f3t_prefetch(G.psiH[1][0] + py);
                            f3t_prefetch(G.psiH[1][1] + py);
                        }
                        if (pz >= 0) f3t_prefetch(G.psiH[2][0] + pz);
                    }
                    if (col_h) {
                        const int px = at_x(cxH, kn), py = at_y(cyH, kn), pz = at_z(cz0, lhzn);
                        if (px >= 0) {
                            f3t_prefetch(G.psiH[0][0] + px);
                            f3t_prefetch(G.psiH[0][1] + px);
                        }
                        if (py >= 0) f3t_prefetch(G.psiH[1][1] + py);
                        if (pz >= 0) f3t_prefetch(G.psiH[2][1] + pz);
                    }
                }
            }
        }
        // plane k's slot completed in the previous iteration (or before the loop); wait for k+1
        fail |= !mbar_wait_bounded(&full[sn], (uint32_t)(rn & 1), F3T_WAIT_CYCLES);
        bool bad;
        if constexpr (MODE == F3T_LEAN_ONLY) {
            // the host's plan and this block's own test agree, or the error word says otherwise
            if (!lean_at(k, z1) && threadIdx.x == 0) atomicOr(err, 4);
            bad = plane(F3tForm<true>{}, k, sc, sn, z0, z1);
        } else {
            bad = lean_at(k, z1) ? plane(F3tForm<true>{}, k, sc, sn, z0, z1)
                                 : plane(F3tForm<false>{}, k, sc, sn, z0, z1);
        }
        if (bad) {
            if (threadIdx.x == 0) atomicOr(err, 1);
            break;
        }
        sc = sn;
        rc = rn;
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

// The grid's arguments in shared memory, at the start of the block's layout: read from there,
// the compiler does not hold the many pointers of the argument block in registers (which spilled).
__device__ __forceinline__ void f3t_args_to_smem(const GridArgs<float> &G, const Fused3Args &A, unsigned char *smem)
{
    const int *src = reinterpret_cast<const int *>(&G);
    int *dst = reinterpret_cast<int *>(smem);
    for (int w = threadIdx.x; w < (int)(sizeof(GridArgs<float>) / 4); w += blockDim.x) dst[w] = src[w];
    src = reinterpret_cast<const int *>(&A);
    dst = reinterpret_cast<int *>(smem + F3T_ARGB);
    for (int w = threadIdx.x; w < (int)(sizeof(Fused3Args) / 4); w += blockDim.x) dst[w] = src[w];
    __syncthreads();
}

// One launch over a list of runs {i0, j0, k0, k1} (tile origin, planes): block b takes items[b].  nd: ring depth
// (the dynamic shared memory holds F3tShape<TY>::smem(nd) bytes).
template <int TY, int MODE>
__global__ void __launch_bounds__(F3tShape<TY>::THREADS, f3t_min_blocks<TY>())
    k_fused3_tma(const __grid_constant__ F3tMaps M, Fused3Args A, GridArgs<float> G, const int4 *__restrict__ items,
                 int nd, int *err)
{
    extern __shared__ __align__(1024) unsigned char f3_smem[];
    f3t_args_to_smem(G, A, f3_smem);
    const int4 it = items[blockIdx.x];
    f3t_tile<TY, MODE>(M.m, *reinterpret_cast<const Fused3Args *>(f3_smem + F3T_ARGB),
                       *reinterpret_cast<const GridArgs<float> *>(f3_smem), it.x, it.y, it.z, it.w, nd, gridDim.x,
                       err, f3_smem);
}

// ---- general runs: the two-kernel form -----------------------------------------------------
// Runs whose planes need CPML psi, the media box or the plane source are updated by two plain
// kernels, one thread per (i, j) column of the run's tile marching its planes (a run {i0 | w << 20,
// j0 | h << 20, k0, k1}: w <= 32 columns from i0, h <= TY rows from j0): new H (from
// the in set, psi in -> out) and then new E (from the out set's new H), with the same device
// functions as the fused pass, so each cell gets the same bits whichever kernel updates it.  The
// H kernel runs beside the lean fused launch; the E kernel after both (it reads the new H of
// neighbouring cells that either of them wrote).  Both are bounded to 1536 threads' worth of
// registers per SM (42 a thread): the extra resident warps hide more of their load latency
// (512^3 dimer scene: 1.80 -> 1.71 ms per step with the H march not unrolled).
// One general run's new H: the block's thread (tx, ty) takes column (i0 + tx, j0 + ty) when it
// lies in the run's w x h tile and the grid.
template <int TY>
__device__ __forceinline__ void f3g_h_run(const Fused3Args &A, const GridArgs<float> &G, int4 it)
{
    const Lay &L = G.L;
    const int i = (it.x & 0xfffff) + (int)threadIdx.x, j = (it.y & 0xfffff) + (int)threadIdx.y;
    const int k0 = it.z, k1 = it.w & 0xfffff;
    if ((int)threadIdx.x >= (it.x >> 20) || (int)threadIdx.y >= (it.y >> 20) || i > L.nx || j > L.ny) return;
    const bool perz = G.per[2] != 0;
    const float *__restrict__ Ex = A.in.f[0];
    const float *__restrict__ Ey = A.in.f[1];
    const float *__restrict__ Ez = A.in.f[2];
    const float dt_mu0 = G.dt_mu0, dhx = G.den_h[0][i], dhy = G.den_h[1][j];
    const int lhx = G.lH[0][i], lhy = G.lH[1][j];
    const int bxH = lhx >= 0 ? lhx + G.L2 * (j - 1) : -1, byH = lhy >= 0 ? (i - 1) + L.nx * lhy : -1;
    const int bz0 = (i - 1) + L.nx * (j - 1), sX = G.L2 * L.ny, sY = L.nx * G.L2, sZ = L.nx * L.ny;
    const int px_ = L.px, pz_ = (int)L.pz;
    int idx = (int)L.off + i + px_ * j + pz_ * k0;   // element offsets < 2^31 (checked by the host)
    for (int k = k0; k <= k1; ++k, idx += pz_) {
        const int kp = (perz && k == L.nz) ? idx - (L.nz - 1) * pz_ : idx + pz_;   // E of plane k + 1
        const float ex_c = Ex[idx], ey_c = Ey[idx], ez_c = Ez[idx];
        const float ez_jp = Ez[idx + px_], ez_ip = Ez[idx + 1], ey_ip = Ey[idx + 1], ex_jp = Ex[idx + px_];
        const float ex_kp = Ex[kp], ey_kp = Ey[kp];
        const float dhz = G.den_h[2][k];
        const int lhz = G.lH[2][k];
        const int px = bxH >= 0 ? bxH + sX * (k - 1) : -1, py = byH >= 0 ? byH + sY * (k - 1) : -1;
        const int pz = lhz >= 0 ? bz0 + sZ * lhz : -1;
        const F3tPsiH q = f3t_load_psiH(G, px, py, pz, true);
        const float hx = f3t_hx(__ldcs(A.in.f[3] + idx), ez_c, ez_jp, ey_c, ey_kp, dhy, dhz, dt_mu0, G, A, j, k, 2, py,
                                pz, q.y0, q.z0);
        const float hy = f3t_hy(__ldcs(A.in.f[4] + idx), ez_c, ez_ip, ex_c, ex_kp, dhx, dhz, dt_mu0, G, A, i, k, 2, px,
                                pz, q.x0, q.z1);
        const float hz = f3t_hz(__ldcs(A.in.f[5] + idx), ey_c, ey_ip, ex_c, ex_jp, dhx, dhy, dt_mu0, G, A, i, j, 2, px,
                                py, q.x1, q.y1);
        __stcs(A.out.f[3] + idx, hx);
        __stcs(A.out.f[4] + idx, hy);
        __stcs(A.out.f[5] + idx, hz);
        if (perz && k == L.nz) {   // periodic ghost plane H(0) = H(nz) (mxll_3D_mod.f90:725-738)
            A.out.f[3][idx - L.nz * pz_] = hx;
            A.out.f[4][idx - L.nz * pz_] = hy;
        }
    }
}

// One general run's new E; then, when G.step_inc is set, the last of the nblk blocks of this
// grid's launch advances the grid's device-loop step counter (this launch ends the pass and holds
// its only reads of the step's scalars).
template <int TY>
__device__ __forceinline__ void f3g_e_run(const Fused3Args &A, const GridArgs<float> &G, int4 it, unsigned nblk)
{
    const Lay &L = G.L;
    const int i = (it.x & 0xfffff) + (int)threadIdx.x, j = (it.y & 0xfffff) + (int)threadIdx.y;
    const int k0 = it.z, k1 = it.w & 0xfffff;
    if ((int)threadIdx.x < (it.x >> 20) && (int)threadIdx.y < (it.y >> 20) && i <= L.nx && j <= L.ny) {
        const float *__restrict__ Hx = A.out.f[3];
        const float *__restrict__ Hy = A.out.f[4];
        const float *__restrict__ Hz = A.out.f[5];
        const float dt_eps0 = G.dt_eps0, dex = G.den_e[0][i], dey = G.den_e[1][j];
        const int lex = G.lE[0][i], ley = G.lE[1][j];
        const int bxE = lex >= 0 ? lex + G.L2 * (j - 1) : -1, byE = ley >= 0 ? (i - 1) + L.nx * ley : -1;
        const int bz0 = (i - 1) + L.nx * (j - 1), sX = G.L2 * L.ny, sY = L.nx * G.L2, sZ = L.nx * L.ny;
        const bool bbc = i >= G.bb0[0] && i <= G.bb1[0] && j >= G.bb0[1] && j <= G.bb1[1];
        const int px_ = L.px, pz_ = (int)L.pz;
        int idx = (int)L.off + i + px_ * j + pz_ * k0;
        // new Hx, Hy of plane k - 1 (plane 0: the periodic image written by the pass, or the zero ghost)
        float hxm = Hx[idx - pz_], hym = Hy[idx - pz_];
        for (int k = k0; k <= k1; ++k, idx += pz_) {
            const float hx = Hx[idx], hy = Hy[idx], hz = Hz[idx];
            const float hz_im = Hz[idx - 1], hy_im = Hy[idx - 1], hz_jm = Hz[idx - px_], hx_jm = Hx[idx - px_];
            const float dez = G.den_e[2][k];
            const int lez = G.lE[2][k];
            float rx, ry, rz, dhxk, dhyk;
            f3t_curl(hx, hy, hz, hz_im, hy_im, hz_jm, hx_jm, hxm, hym, dex, dey, dez, rx, ry, rz, dhxk, dhyk);
            hxm = hx;
            hym = hy;
            float ex = __ldcs(A.in.f[0] + idx), ey = __ldcs(A.in.f[1] + idx), ez = __ldcs(A.in.f[2] + idx);
            f3t_e_general(ex, ey, ez, rx, ry, rz, dhxk, dhyk, hx, hy, hz, hz_im, hy_im, hz_jm, hx_jm, i, j, k,
                          bxE >= 0 ? bxE + sX * (k - 1) : -1, byE >= 0 ? byE + sY * (k - 1) : -1,
                          lez >= 0 ? bz0 + sZ * lez : -1, __ldg(G.bE[2] + k), __ldg(G.cE[2] + k), bbc, dt_eps0, G);
            __stcs(A.out.f[0] + idx, ex);
            __stcs(A.out.f[1] + idx, ey);
            __stcs(A.out.f[2] + idx, ez);
        }
    }
    if (G.step_inc) {
        __syncthreads();
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            __threadfence();
            if (atomicAdd((unsigned *)G.step_done, 1u) == nblk - 1) {
                *G.step_done = 0;
                *G.step_inc += 1;
                __threadfence();
            }
        }
    }
}

template <int TY>
__global__ void __launch_bounds__(32 * TY, 1536 / (32 * TY)) k_f3g_h(Fused3Args A, GridArgs<float> G, const int4 *__restrict__ items)
{
    f3g_h_run<TY>(A, G, items[blockIdx.x]);
}

template <int TY>
__global__ void __launch_bounds__(32 * TY, 1536 / (32 * TY)) k_f3g_e(Fused3Args A, GridArgs<float> G, const int4 *__restrict__ items)
{
    f3g_e_run<TY>(A, G, items[blockIdx.x], gridDim.x);
}

// Batched general runs of several grids: items[b].w carries the run's grid (k1 | g << 20); the
// grid's arguments are read from its table entry.
template <int TY>
__global__ void __launch_bounds__(32 * TY, 1536 / (32 * TY)) k_f3g_h_batch(const F3tBatchGrid *__restrict__ grids,
                                                                        const int4 *__restrict__ items)
{
    const int4 it = items[blockIdx.x];
    const F3tBatchGrid &B = grids[it.w >> 20];
    f3g_h_run<TY>(B.A, B.G, it);
}

template <int TY>
__global__ void __launch_bounds__(32 * TY, 1536 / (32 * TY)) k_f3g_e_batch(const F3tBatchGrid *__restrict__ grids,
                                                                        const int4 *__restrict__ items)
{
    const int4 it = items[blockIdx.x];
    const F3tBatchGrid &B = grids[it.w >> 20];
    f3g_e_run<TY>(B.A, B.G, it, (unsigned)B.n_gen);
}

// ---- batched: the fused pass of several grids in one launch ----------------------------------
// Block b takes block b - item0 of the grid whose item range holds it (grids in the order of the
// table, largest first, so that the small grids' blocks fill the tail); the grid's arguments are
// copied into shared memory first.  Each grid computes exactly what its own k_fused3_tma does
// (same f3t_tile arithmetic; every tile shape gives the same bits).
template <int TY>
__global__ void __launch_bounds__(F3tShape<TY>::THREADS, f3t_min_blocks<TY>())
    k_fused3_batch(const F3tBatchGrid *__restrict__ grids, int n, int nd, int *err)
{
    extern __shared__ __align__(1024) unsigned char f3_smem[];
    const long long b = blockIdx.x;
    int lo = 0, hi = n - 1;                    // last grid with item0 <= b
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (grids[mid].item0 <= b) lo = mid;
        else hi = mid - 1;
    }
    const F3tBatchGrid &B = grids[lo];
    f3t_args_to_smem(B.G, B.A, f3_smem);
    const GridArgs<float> *sG = reinterpret_cast<const GridArgs<float> *>(f3_smem);
    const Fused3Args *sA = reinterpret_cast<const Fused3Args *>(f3_smem + F3T_ARGB);
    const long long t = b - B.item0;
    const int bx = (int)(t % B.tx), by = (int)((t / B.tx) % B.ty), bz = (int)(t / ((long long)B.tx * B.ty));
    const int k0 = 1 + bz * B.kch, k1 = min(sG->L.nz, k0 + B.kch - 1);
    f3t_tile<TY, F3T_MIXED>(B.m, *sA, *sG, 1 + 32 * bx, 1 + TY * by, k0, k1, nd,
                            (unsigned)((long long)B.tx * B.ty * B.tz), err,
                            f3_smem);
}

// Batched lean runs of several grids (items[b] = {i0, j0, k0, k1 | g << 20}): the grid's
// arguments are copied into shared memory; a grid that has general runs leaves its step counter
// to their E launch.
template <int TY>
__global__ void __launch_bounds__(F3tShape<TY>::THREADS, f3t_min_blocks<TY>())
    k_fused3_batch_lean(const F3tBatchGrid *__restrict__ grids, const int4 *__restrict__ items, int nd, int *err)
{
    extern __shared__ __align__(1024) unsigned char f3_smem[];
    const int4 it = items[blockIdx.x];
    const F3tBatchGrid &B = grids[it.w >> 20];
    f3t_args_to_smem(B.G, B.A, f3_smem);
    GridArgs<float> *sG = reinterpret_cast<GridArgs<float> *>(f3_smem);
    if (B.n_gen > 0 && threadIdx.x == 0) {
        sG->step_inc = nullptr;
        sG->step_done = nullptr;
    }
    __syncthreads();
    const Fused3Args *sA = reinterpret_cast<const Fused3Args *>(f3_smem + F3T_ARGB);
    f3t_tile<TY, F3T_LEAN_ONLY>(B.m, *sA, *sG, it.x, it.y, it.z, it.w & 0xfffff, nd, (unsigned)B.n_lean, err,
                                f3_smem);
}

}  // namespace omx
