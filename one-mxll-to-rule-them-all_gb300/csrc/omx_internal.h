// omx_internal.h -- device-side data layout and kernel argument blocks.
//
// HBM layout (every field component, both precisions):
//   element (i, j, k) lives at  off + i + px*j + pz*k  with i in [0, nx+1], j in [0, ny+1],
//   k in [0, nz+1] (2D: k == 0; 1D: j == k == 0 and the only axis is i).  px is a multiple
//   of 32 elements and off is chosen so that element i == 1 of every row starts on a 128-byte
//   boundary: a warp reading 32 consecutive interior cells touches exactly one 128-byte line
//   per row (FP32) or two (FP64).  The ghost layers i,j,k == 0 and n+1 hold the reference's
//   boundary values (zero for PEC); periodic axes are closed by index remapping in the
//   kernels instead of ghost copies.
//
// CPML auxiliary fields (psi) exist only inside the absorbing slabs: for each axis a and each
// field kind (E or H) two components, stored over 2*(npml-1) layers (low face layers first,
// then high face) x the two transverse axes, ordered so that consecutive i are consecutive in
// memory.  Material ids (uint8, one per component) and the auxiliary-differential-equation
// state exist only inside the bounding box of non-vacuum cells.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace omx {

enum KernelClass { KC_H = 0, KC_E = 1, KC_EMIT = 2, KC_SRC = 3, KC_DET = 4, KC_N = 5 };

struct Lay {
    int dims;
    int nx, ny, nz;   // interior cells per axis (1D: nx = N, ny = nz = 1)
    int px;           // row pitch in elements
    long long pz;     // plane pitch in elements
    long long off;    // element offset of (0,0,0)
};

// Scalar that is either an immediate value or tab[*step * stride] on the device (for graphs:
// the run's per-step table is step-major, one row of `stride` scalars per step).
struct StepParam {
    double val;
    const double *tab;
    const int *step;
    int stride;
};

enum ClsType { CLS_PLAIN = 0, CLS_DRUDE = 1, CLS_DL = 2 };

template <class R> struct ClsR {
    int type;      // ClsType
    int medium;    // index into the medium table (ADE classes)
    R coef;        // dt_eps0 * eps_inv (plain classes)
    R pad;
};

template <class R> struct MedR {
    R A1, A2, C1, C2, C3, C4;
    R al[8], be[8], ga[8], B1[8], B2[8];
    int np;
    int pad;
};

template <class R> struct GridArgs {
    Lay L;
    R dt_mu0, dt_eps0;
    R dr;              // used by the exact path's CPML division
    int per[3];        // periodic axes
    int npml, L2;      // L2 = 2*(npml-1) psi layers per axis
    const R *den_e[3], *den_h[3];
    const R *bE[3], *cE[3], *bH[3], *cH[3];
    const short *lE[3], *lH[3];
    R *psiE[3][2], *psiH[3][2];
    // media bounding box (1-based inclusive); empty when bb1 < bb0
    int bb0[3], bb1[3], bbd[3];
    long long bbV;
    const uint8_t *mat[3];
    const ClsR<R> *cls;
    const MedR<R> *med;
    R *ade;            // [comp][slot][bbV], slot 0 = PD, 1 = E_old, 2+p = PL, 2+P+p = PL_old
    int P;             // poles per cell in the ADE state
    int mode2d;        // 1 TMz, 2 TEz
    // dispersive component-cells, updated by their own kernel before the bulk E pass:
    // (i, j, k, component) and the media-box index of each
    int ade_n;
    const int4 *ade_ent;
    const int *ade_b;
    // device-loop step counter, advanced by the first kernel of each step (null outside omx_run);
    // the fused 3D pass advances it when its last block finishes (step_done counts the blocks)
    int *step_inc;
    int *step_done;
    // planes (3D) or rows (2D) marched per thread by the unfused kernels; 0 = default
    int march;
    // a plane soft source added by the 3D bulk E pass to E_old before the update, as k_plane
    // does before the pass (pl_on = 0: none); the host enables it only when no plane cell is
    // dispersive
    int pl_on, pl_comp, pl_axis, pl_index;
    double pl_c_src;
    StepParam pl_amp;
};

template <class R> struct FieldPtrs {
    R *f[6];           // Ex, Ey, Ez, Hx, Hy, Hz
};

struct JState {
    int np;            // number of J points
    double *J[3], *Jo[3], *dJ[3];
};

struct InjArgs {
    int n;
    const long long *eidx;
    const int *comp;
    const int *sa, *sb;
    int avg;           // 1: 0.5*(J(i) + J(i+1)) average; 0: J(i) only
};

struct SrcArgs {
    int n;
    const long long *eidx;
    const double *ka, *kb;
    int comp;          // 0..2
    int avg;
    double c_src;
};

struct PlaneArgs {
    int comp, axis, index;
    double c_src;
};

struct EmitArgs {
    int n, model, npar, nst, dims, mode2d;
    const int *ci, *cj, *ck;
    const double *par;
    const double *rates;      // (1/T1, 1/T2) per emitter, formed at group creation
    double *rho, *E, *dipole, *dPdt;
    double dt, h2, h6;        // dt, dt/2, dt/6
    // 0: dPt_dt = (new - old) / dt, the reference's division (FP64 fields); else (new - old) * inv_dt,
    // 1/dt rounded once (FP32 fields: within an ulp of the quotient, without an FP64 division)
    double inv_dt;
    const int *only_if;       // optional: run only while *only_if != 0 (the closure's fallback flag)
};

struct ScatArgs {
    int np, c0, c1;
    const int *win;
    const double *wk;
    const double *dPdt;
    double dt;
    double inv_dt;            // as EmitArgs::inv_dt, for dJ = (J - J_old) / dt
};

struct DetArgs {
    int n;
    const int *field;      // 0..5
    const int *nt;
    const double *w;
    const long long *t0, *t1, *t2, *t3;
    double *rec;           // [capacity][n]
    double *times;
    // running Fourier transforms of every sample (FP64): re/im[k][s] += w * v * (cos, -sin)(omega_k t)
    int n_freq;
    const double *omega;
    double *dft_re, *dft_im;
    double dft_w;
};

// ---- launchers (instantiated in omx_kernels_fast.cu / omx_kernels_exact.cu) ------------------
template <class R> void launch_h(const FieldPtrs<R> &F, const GridArgs<R> &G, void *stream);
template <class R> void launch_e(const FieldPtrs<R> &F, const GridArgs<R> &G, void *stream);
template <class R> void launch_src(const FieldPtrs<R> &F, const SrcArgs &S, StepParam amp, void *stream);
template <class R> void launch_plane(const FieldPtrs<R> &F, const Lay &L, const PlaneArgs &P, StepParam amp, void *stream);
template <class R> void launch_inject(const FieldPtrs<R> &F, const JState &J, const InjArgs &I, StepParam time,
                                      StepParam t_skip, double dt_eps0, void *stream);
template <class R> void launch_emit(const FieldPtrs<R> &F, const Lay &L, const EmitArgs &A, StepParam move, void *stream);
void launch_scatter(const JState &J, const ScatArgs &S, StepParam move, void *stream);
template <class R> void launch_sample(const FieldPtrs<R> &F, const DetArgs &D, StepParam slot, StepParam time, void *stream);
void launch_step_advance(int *step, void *stream);
// FP32 fused TMz step: reads the in buffers, writes the out buffers (see omx_fused2d.cuh)
struct Fused2Args {
    const float *ez_in, *hx_in, *hy_in;
    float *ez_out, *hx_out, *hy_out;
    const float *psi_hyx_in, *psi_hxy_in;   // x-face psi of Hy, y-face psi of Hx (old)
    float *psi_hyx_out, *psi_hxy_out;
    float *psi_ezx, *psi_ezy;               // E psi, updated in place
    int *err;                               // device error word (bit 0: a bulk-copy wait ran out)
    // per-row y coefficients, two float4 per row j = 0..ny+1: (den_h, den_e, bH, cH) and
    // (bE, cE, H psi layer, E psi layer) with the layers stored as int bit patterns
    const float4 *rowc;
};
// form: 0 register prefetch, 4/5/6/8 bulk-copy ring depth, 14/15/16 ring depth 4/5/6 with a
// dedicated copy warp; < 0 the default
void launch_fused_tmz(const Fused2Args &A, const GridArgs<float> &G, int form, void *stream);
// FP32 fused 3D step (k_fused3_tma): in / out buffer sets, the out set's H psi
struct Fused3Args {
    FieldPtrs<float> in, out;
    float *psiH_out[3][2];   // H psi of the out set (the in set's is GridArgs::psiH)
};
// tensor maps of the in set's six components (Ex, Ey, Ez, Hx, Hy, Hz) for the fused 3D pass:
// coordinate x = 0 is element i = -3 of a row (so x = 32 t is 16-byte aligned and reaches the
// halo column i = 32 t), y = j, z = k; box {40, ty + 2, 1}
struct F3tMaps {
    CUtensorMap m[6];
};
// one grid of a batched fused 3D pass: its in set's tensor maps, arguments and block range
struct F3tBatchGrid {
    CUtensorMap m[6];
    GridArgs<float> G;
    Fused3Args A;
    long long item0;         // first block of this grid in the launch
    int tx, ty, tz, kch;     // tiles along x (32 cells), y (tile rows), z (kch planes)
    int n_gen, n_lean;       // the grid's general and lean runs in the run lists of a split launch
};
constexpr int F3T_KMAX = 128;   // planes per block of the fused 3D pass at most
constexpr int F3T_GEN_KCH = 8;  // planes per run of the fused 3D pass's general runs at most
constexpr int F3T_MEDIA_KCH = 1;   // the same in the media box's planes when it holds dispersive cells
// a fused 3D form is ring depth x 100 + tile rows (8 or 16); depth 0 and form <= 0 are defaults
constexpr int F3T_RING_DEFAULT = 4;   // plane slots in a block's ring
constexpr int F3T_RING_MAX = 16;
inline int f3t_rows(int form) { return form > 0 && form % 100 == 16 ? 16 : 8; }
inline int f3t_ring(int form) { return form >= 200 ? form / 100 : F3T_RING_DEFAULT; }
// dynamic shared memory of a fused 3D block of this form (bytes)
int f3t_smem_bytes(int form);
bool encode_f3t_maps(F3tMaps *M, const FieldPtrs<float> &in, const Lay &L, int ty);
// The fused 3D pass's lean runs (no CPML, media or plane source at them) in one launch over n
// runs {bx, by, k0, k1} (tile, planes k0..k1) of one grid.  form: ring depth x 100 + tile rows;
// err: the device error word.  The launch advances the device-loop step counter when
// G.step_inc is set.
cudaError_t launch_fused3t_lean(const F3tMaps &M, const Fused3Args &A, const GridArgs<float> &G, int form,
                                const int4 *items, int n, int *err, void *stream);
// The general runs of the fused 3D pass through the two plain kernels: new H (e_half = false;
// reads the in set only) or new E (e_half = true; after every new H of the step is written; it
// advances the device-loop step counter when G.step_inc is set).
cudaError_t launch_fused3t_general(const Fused3Args &A, const GridArgs<float> &G, int form, const int4 *items, int n,
                                   bool e_half, void *stream);
// The batched fused pass split by plane form: every grid's general runs through the two plain
// kernels (new H, then new E after the lean runs) and every grid's lean runs in one launch; run
// lists as the single-grid ones with the grid's table index in k1's high bits (k1 | g << 20).
// parts: 1 the general runs' new H, 2 the lean runs, 4 the general runs' new E (which reads the
// new H of both), launched in that order; 1 and 2 may run on two streams at once.
cudaError_t launch_fused3t_batch_split(const F3tBatchGrid *grids, const int4 *gen, int ngen, const int4 *lean, int nlean,
                                       int form, int parts, int *err, void *stream);
// the batched pass over n grids (device table, largest grid first) with `blocks` blocks in all
cudaError_t launch_fused3t_batch(const F3tBatchGrid *grids, int n, long long blocks, int form, int *err,
                                 void *stream);
void launch_ade_post(const FieldPtrs<float> &Fin, const FieldPtrs<float> &Fout, const GridArgs<float> &G, void *stream);
// The work after a fused pass in one launch: the dispersive cells (as launch_ade_post), one
// plane source (as launch_plane) and the emitter current (as launch_inject).  Only for lists
// that write disjoint E words (the host checks), so the result equals the separate launches.
struct PostArgs {
    int nb_ade, nb_plane, nb_inj;   // blocks of 128 threads per list
    int plane_n0, plane_cells;      // plane cells along the first in-plane axis, in all
    PlaneArgs P;
    StepParam amp;
    InjArgs I;
    JState J;
    StepParam time, tskip;
    double dt_eps0;
};
void launch_post_fused(const FieldPtrs<float> &Fin, const FieldPtrs<float> &Fout, const GridArgs<float> &G,
                       const PostArgs &Q, void *stream);
void launch_flush(float *buf, long long n, void *stream);
// FP64 electromagnetic energy of the interior: 0.5 * dV * sum(eps0 E^2 + mu0 H^2) over the fields
// present (vacuum constants; each component over its own interior index range)
template <class R> void launch_field_energy(const FieldPtrs<R> &F, const Lay &L, const int *used, double eps0,
                                            double mu0, double dV, double *out, void *stream);

// ---- learned closure: plain-propagator work that must round like the q-group kernel ------------
// training trajectories: per trajectory q, E(t_s) = amp * sum_k c_k cos(w_k t_s + phi_k) with
// t_s = s * dt (drive[q] = amp, then K triples c, w, phi); the emitter (params[q], npar values)
// starts in the ground state and is advanced by the q-group's RK4 with E held over each step.
struct ClTrajArgs {
    int n, T, K, model, npar;
    double dt, e_scale, d_scale;
    const double *params, *drive;
    float *e, *d;            // [n][T]: E(t_s) / e_scale and the dipole after step s / d_scale
};
void launch_cl_trajectories(const ClTrajArgs &A, void *stream);

// deployment of a trained closure in a q-group (device-side control, so that a captured graph
// needs no host decision): the state block and the per-group arguments
constexpr int CL_WIN = 32;
struct ClDevState {
    int cl_step;          // closure steps taken (the window ring's head is cl_step % CL_WIN)
    int use_plain;        // 1 once the spot-check failed: the plain propagator runs from then on
    int skip_nn;          // 1 when the network does not run this step (no q-step, or use_plain)
    int reseed;           // 1 on the step the fallback happened (density matrices re-seeded)
    int checks, fallback_step, steps_since_check;
    int plain_now;        // use_plain as it was when this step began (the plain kernel's switch)
    unsigned long long err_bits, scale_bits;   // running max |closure - plain|, max |plain| (>= 0)
    double last_err;      // error of the last completed check window
};
struct ClDeploy {
    int n, n_sub, check_every;
    double e_scale, d_scale, tol;
    float *win;           // [n][CL_WIN] scaled field history on the dipole axis
    float *hst;           // [n][128] GRU state
    uint16_t *xh;         // [n][160] network input (BF16)
    float *G, *Y;         // [n][512] gate pre-activations, [n][16] read-out
    uint16_t *hb, *a1, *a2, *a3;   // [n][128], [n][256] x 3 layer outputs (BF16)
    const int *sub;       // [n_sub] emitters of the spot-check subset
    const int *sub_of;    // [n] subset slot of each emitter, or -1
    double *sub_rho;      // [n_sub][nst] their plain density matrices
    ClDevState *st;
    int *err;             // error word of the owning context (tensor-core pipeline waits)
};
template <class R> void launch_cl_gather(const FieldPtrs<R> &F, const Lay &L, const EmitArgs &A, const ClDeploy &D,
                                         StepParam move, void *stream);
void launch_cl_subset_check_reseed(const EmitArgs &A, const ClDeploy &D, void *stream);

// ---- batched multi-grid launches (3D): one launch per pass over several grids ----------------
template <class R> struct BatchGrid {
    GridArgs<R> G;
    FieldPtrs<R> F;
    long long tile0;   // first tile of this grid in the concatenated tile list
    int tx, ty;        // tiles along x (32 cells) and y (4 cells); along z: kch planes each
};
template <class R> struct BatchSrc {     // one radial source of one grid
    FieldPtrs<R> F;
    SrcArgs S;
    StepParam amp;
    long long p0;      // first point of this entry in the concatenated point list
};
template <class R> struct BatchDet {     // the detectors of one grid
    FieldPtrs<R> F;
    DetArgs D;
    StepParam slot, time;
    long long p0;
};
// pass 0: H, pass 1: bulk E (dispersive cells before it with launch_ade)
template <class R> void launch_batch3(int pass, const BatchGrid<R> *grids, int n, long long total, int kch,
                                      int blocks, void *stream);
template <class R> int batch3_blocks();   // persistent grid: SMs x resident blocks
template <class R> void launch_ade(const FieldPtrs<R> &F, const GridArgs<R> &G, void *stream);
template <class R> void launch_src_batch(const BatchSrc<R> *e, int n, long long total, void *stream);
template <class R> void launch_sample_batch(const BatchDet<R> *e, int n, long long total, void *stream);

}  // namespace omx
