/*
 * omx_oracle.h -- CPU FP64 restatement of the OMxRTA time-domain hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the checker for the GPU library:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 * The product path (libomx_gpu.so) never links or calls it.
 *
 * PARITY UNPINNED against the reference itself: the reference is Fortran 2008,
 * no Fortran compiler exists in the build container, the reference ships no
 * tests, golden vectors or fixtures, and its only emitter backend (DFTB+) is
 * an un-vendored external library with no pinned version.  The oracle is
 * pinned instead by analytic known-answer tests (Yee dispersion relation,
 * closed-cavity energy conservation, CPML reflection, ADE z-transform,
 * Rabi/T1/T2 Bloch dynamics) and by line-by-line restatement of the
 * reference's arithmetic, including its single-precision literal quirks.
 *
 * Every function cites the reference file:line it restates (paths relative to
 * the reference project root, src/FDTD/).
 *
 * Array conventions follow the reference exactly: Fortran column-major with
 * the reference's lower bounds (e.g. Ex(0:nx, 1:ny+1, 1:nz+1)).
 */
#ifndef OMX_ORACLE_H
#define OMX_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* constants_mod.f90 enum codes */
enum { ORC_CLOSE = 1, ORC_PERIODIC = 2, ORC_CPML = 3 };
enum { ORC_TMZ = 1, ORC_TEZ = 2 };
enum { ORC_NONE_MEDIUM = 0, ORC_DIELECTRIC = 1, ORC_DRUDE = 2, ORC_DL = 3 };
enum { ORC_EX = 1, ORC_EY, ORC_EZ, ORC_HX, ORC_HY, ORC_HZ };
enum { ORC_Q_MATERIAL = 1, ORC_Q_SINGLE = 2 };
enum { ORC_POINT = 1, ORC_LINE_X, ORC_LINE_Y, ORC_LINE_Z, ORC_PLANE_XY, ORC_PLANE_YZ,
       ORC_PLANE_ZX, ORC_VOLUME };

#define ORC_MAX_POLES 8

/* Constants with the reference's literal precision (constants_mod.f90). */
typedef struct {
    double pi0, c0, eps0, mu0;
    double sec_to_au, C_to_au, kg_to_au, m_to_au;
    double nm_to_au, au_to_nm, ev_to_au, au_to_ev, Debye_to_au, fs_to_au, au_to_fs;
    double alphaCPML, kappaCPML;
    double aBH[4];
    double sig_to_au;
} orc_constants;
void orc_get_constants(orc_constants *out);

/* TClassicalMedium coefficients (classical_medium_mod.f90:6-37). */
typedef struct {
    int    medium_type;
    int    n_poles;
    double eps_r;
    double A1, A2, C1, C2, C3, C4;
    double alpha_k[ORC_MAX_POLES], beta_k[ORC_MAX_POLES], gamma_k[ORC_MAX_POLES];
    double B1_k[ORC_MAX_POLES], B2_k[ORC_MAX_POLES];
    double omegaD, GammaD, omegaP;
    double omegaP_i[ORC_MAX_POLES], GammaP_i[ORC_MAX_POLES], AP_i[ORC_MAX_POLES];
} orc_medium;

/* init_classical_medium (classical_medium_mod.f90:46-104). omegaD/GammaD in a.u. */
void orc_medium_dielectric(double eps_r, orc_medium *m);
void orc_medium_drude(double omegaD_au, double GammaD_au, double eps_r, double dt, orc_medium *m);
/* library materials "Ag" "Al" "Au" (get_DL_library_data, :125-199); returns 0 ok, -1 unknown */
int  orc_medium_dl_library(const char *material, double eps_r, double dt, orc_medium *m);
/* custom Drude-Lorentz poles in eV (extension: same ADE math, A_k = f_k * wp^2, omegaD = wp) */
void orc_medium_dl_custom(double eps_inf, double wp_ev, double gamma_ev, int n_poles,
                          const double *pole_ev, const double *strength,
                          const double *width_ev, double dt, orc_medium *m);

/* CPML tables (mxll_3D_mod.f90:282-318): be,ce[npml], bh,ch[npml-1],
 * kappae[npml], kappah[npml-1]. */
void orc_cpml_tables(int npml, double dr, double dt, double *be, double *ce, double *bh,
                     double *ch, double *kappae, double *kappah);

/* Media map from voxel lists (read_init_media_{1D,2D,3D}).  voxel coords in nm,
 * media_map written in Fortran order with shape (nx,ny,nz,3)/(nx,ny,3)/(nz). */
int orc_media_map_3d(int nx, int ny, int nz, double dr, int n_media, const int *n_vox,
                     const double *vox_xyz_nm, int32_t *media_map);
int orc_media_map_2d(int nx, int ny, double dr, int n_media, const int *n_vox,
                     const double *vox_xy_nm, int32_t *media_map);
int orc_media_map_1d(int nz, double dr, int n_media, const int *n_vox,
                     const double *vox_x_nm, int32_t *media_map);

/* ---------------------------------------------------------------------------------------- */
/* Grid (TMxll_1D/2D/3D).                                                                  */
typedef struct orc_grid orc_grid;

orc_grid *orc_grid_create(int dims, int nx, int ny, int nz, int npml, const int boundaries[3],
                          int mode, double dt, double dr);
void orc_grid_destroy(orc_grid *g);
/* media: n_media descriptors; media_map Fortran order as produced by orc_media_map_*;
 * eps arrays (x,y,z, Fortran (nx,ny,nz)) may be NULL -> reference rule (read_init_media_*). */
int  orc_grid_set_media(orc_grid *g, int n_media, const orc_medium *media,
                        const int32_t *media_map, const double *eps_x, const double *eps_y,
                        const double *eps_z);
void orc_grid_set_time(orc_grid *g, double time, double t_skip);
void orc_propagate_H(orc_grid *g);
void orc_propagate_E(orc_grid *g);
/* read/write a field including ghost planes, Fortran order over the reference bounds.
 * field codes ORC_EX..ORC_HZ; returns element count or -1 */
long orc_field_size(const orc_grid *g, int field);
long orc_field_get(const orc_grid *g, int field, double *out);
long orc_field_set(orc_grid *g, int field, const double *in);
/* reference bounds of a field: lo[3], hi[3] */
int  orc_field_bounds(const orc_grid *g, int field, int lo[3], int hi[3]);
void orc_get_den(const orc_grid *g, double *den_e, double *den_h); /* 3 x nmax each, axis-major */

/* ---------------------------------------------------------------------------------------- */
/* Sources (source_mod.f90, interactions_mod.f90:21-163).                                  */
typedef struct {
    char   dir;            /* 'x' 'y' 'z' */
    double j_amp, w0, t0, tau, t_init, t_final, phase;  /* a.u. */
    double r0[3];          /* a.u. */
    double rad;            /* a.u. */
    double chirp;          /* extension: d(omega)/dt in a.u.; 0 -> reference */
} orc_source_desc;
typedef struct orc_source orc_source;
orc_source *orc_source_create(const orc_grid *g, const orc_source_desc *d);
void orc_source_destroy(orc_source *s);
void orc_source_update(orc_source *s, double time);              /* update_source :106-132 */
void orc_source_interactions(orc_grid *g, orc_source **s, int n); /* :21-163 */
int  orc_source_kernel(const orc_source *s, double *ker, int *n_ker);

/* Plane-wave soft source (extension; no reference counterpart): E_comp on the plane
 * axis==plane_axis at index plane_idx gets += c_src * j_amp * env * cos. */
typedef struct {
    int    comp;           /* 1..3 */
    int    plane_axis;     /* 1..3 */
    int    plane_idx;
    double j_amp, w0, t0, tau, t_init, t_final, phase, chirp;
} orc_plane_source_desc;
void orc_plane_source_apply(orc_grid *g, const orc_plane_source_desc *d, double time);

/* ---------------------------------------------------------------------------------------- */
/* Few-level density-matrix emitters (new model behind TQ_sys_base) and q-groups.         */
enum { ORC_EMITTER_2LEVEL = 1, ORC_EMITTER_3LEVEL = 2 };
typedef struct orc_qgroup orc_qgroup;
/* params per emitter: 2-level [w0, mu, T1, T2, ux, uy, uz]
 *                     3-level [e1, e2, mu1, mu2, T1, T2, ux, uy, uz]  (a.u.) */
orc_qgroup *orc_qgroup_create(const orc_grid *g, int group_type, int model, int n_systems,
                              const int32_t *cell /* n x dims, 1-based */, const double *params,
                              double density, double dt_q);
void orc_qgroup_destroy(orc_qgroup *q);
void orc_send_E_to_J(const orc_grid *g, orc_qgroup *q);          /* interactions_mod:534-695 */
void orc_td_propagate_q_group(orc_qgroup *q, int tq_step);       /* q_group_mod:802-818 */
void orc_send_J_to_E(orc_grid *g, orc_qgroup *q);                /* interactions_mod:1046-1220 */
void orc_qgroup_read(const orc_qgroup *q, double *dipole, double *dPt_dt, double *efield,
                     double *rho);
int  orc_qgroup_state_size(const orc_qgroup *q);
/* single-emitter propagation (RK4 on the Lindblad equation) for KAT tests */
void orc_emitter_step(int model, const double *params, double *rho, double E_u, double dt);

/* ---------------------------------------------------------------------------------------- */
/* Detector sampling stencils (write_fields_subs_mod.f90).                                  */
/* idx: nd x dims (Fortran (nd,dims) order); out: nd values */
void orc_sample(const orc_grid *g, int detector_type, int field, int nd, const int32_t *idx,
                double *out);

/* ---------------------------------------------------------------------------------------- */
/* Whole time loop (mxim_mxll.f90:92-132) over a prepared scene, for the CPU baseline.     */
typedef struct {
    orc_grid       *grid;
    int             n_src;
    orc_source    **src;
    int             n_plane;
    orc_plane_source_desc *plane;
    int             n_groups;
    orc_qgroup    **groups;
    int             n_skip_steps;
    int             t_det_print;
    int             n_det;
    const int      *det_type;
    const int      *det_field;
    const int      *det_nd;
    const int32_t **det_idx;
    double         *det_out;   /* (n_records x total_points) or NULL */
    int             tq_step_old;
    double          t_skip;
    int             record;
} orc_scene;
/* runs steps tt = tt0 .. tt0+nsteps-1 (1-based as the reference) */
void orc_run(orc_scene *s, int tt0, int nsteps);

int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
