/*
 * omx_gpu.h -- C-ABI of the GB300 (sm_103a) library for OMxRTA's time-domain hot path.
 *
 * The entry points replace the bodies behind the reference's plugin interfaces
 * (paths relative to the reference project root):
 *   TMxll        src/FDTD/mxll_base_mod.f90:7-69   (init / kill / td_propagate_H_field /
 *                                                   td_propagate_E_field)
 *   TQ_sys_base  src/FDTD/q_sys_base_mod.f90:7-71  (td_propagate, batched per q-group)
 *   free routines called by the driver src/FDTD/mxim_mxll.f90:107-126:
 *                source_interactions, send_E_to_J_ranks, td_propagate_q_group,
 *                send_J_to_E_ranks, write_detectors_outputs (sampling only).
 *
 * Conventions
 *   - Every call returns an int status (OMX_OK == 0).  The reference stops the program
 *     on errors; a Fortran caller maps a non-zero status to `error stop`.
 *   - All device memory is owned by the library; callers pass host pointers.
 *   - Array arguments use the reference's Fortran layout (column-major, first index
 *     fastest) and the reference's array bounds, so a Fortran caller passes its own
 *     arrays unchanged.
 *   - Units are atomic units, as inside the reference after its input conversion.
 *   - One host thread per context; calls on one context are not re-entrant.
 *   - There is no CPU fallback: omx_create fails when no CUDA device is usable.
 */
#ifndef OMX_GPU_H
#define OMX_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------------- */
#define OMX_OK 0
#define OMX_ERR_ARG 1      /* invalid argument or unsupported combination */
#define OMX_ERR_CUDA 2     /* CUDA runtime error (message in omx_last_error) */
#define OMX_ERR_STATE 3    /* call out of order (e.g. media after the first step) */
#define OMX_ERR_NOMEM 4    /* device allocation failed */
#define OMX_ERR_NODEV 5    /* no usable CUDA device */

/* ---- enum codes: identical to constants_mod.f90:52-105 ----------------------------------- */
#define OMX_CLOSE_BOUNDARIES 1
#define OMX_PERIODIC_BOUNDARIES 2
#define OMX_CPML_BOUNDARIES 3

#define OMX_TMZ_2D_MODE 1
#define OMX_TEZ_2D_MODE 2

#define OMX_NONE_MEDIUM 0
#define OMX_DIELECTRIC_MEDIUM 1
#define OMX_DRUDE_MEDIUM 2
#define OMX_DL_MEDIUM 3

#define OMX_EX_FIELD 1
#define OMX_EY_FIELD 2
#define OMX_EZ_FIELD 3
#define OMX_HX_FIELD 4
#define OMX_HY_FIELD 5
#define OMX_HZ_FIELD 6

#define OMX_POINT_DETECTOR 1
#define OMX_LINE_X_DETECTOR 2
#define OMX_LINE_Y_DETECTOR 3
#define OMX_LINE_Z_DETECTOR 4
#define OMX_PLANE_XY_DETECTOR 5
#define OMX_PLANE_YZ_DETECTOR 6
#define OMX_PLANE_ZX_DETECTOR 7
#define OMX_VOLUME_DETECTOR 8

#define OMX_Q_MATERIAL 1
#define OMX_Q_SINGLE 2

/* ---- library-specific codes ---------------------------------------------------------------- */
#define OMX_PREC_FP64 0    /* plain FP64 path: reference arithmetic, no FMA contraction */
#define OMX_PREC_FP32 1    /* fused FP32 path: FP32 state, FP64-precomputed coefficients */

#define OMX_EMITTER_TWO_LEVEL 1    /* params: w0, mu, T1, T2, ux, uy, uz           (7) */
#define OMX_EMITTER_THREE_LEVEL 2  /* params: e1, e2, mu1, mu2, T1, T2, ux, uy, uz (9) */

#define OMX_MAX_POLES 8

typedef struct omx_ctx omx_ctx;

/* TMxll%init arguments (mxll_base_mod.f90:41-57) plus the precision of the GPU path. */
typedef struct {
    int    dimensions;     /* 1, 2 or 3 */
    int    grid_Ndims[3];  /* cells per axis (1D: grid_Ndims[0] is the only axis) */
    int    npml;           /* CPML thickness in cells (>= 2 when any axis is CPML) */
    int    boundaries[3];  /* OMX_*_BOUNDARIES per axis */
    int    mode;           /* 2D only: OMX_TMZ_2D_MODE or OMX_TEZ_2D_MODE */
    int    precision;      /* OMX_PREC_FP64 or OMX_PREC_FP32 */
    double dt;             /* a.u. */
    double dr;             /* a.u. */
} omx_grid_desc;

/* TClassicalMedium coefficients (classical_medium_mod.f90:6-37). */
typedef struct {
    int    medium_type;    /* OMX_*_MEDIUM */
    int    n_poles;        /* Drude-Lorentz poles (<= OMX_MAX_POLES) */
    double eps_r;
    double A1, A2, C1, C2, C3, C4;
    double alpha_k[OMX_MAX_POLES], beta_k[OMX_MAX_POLES], gamma_k[OMX_MAX_POLES];
    double B1_k[OMX_MAX_POLES], B2_k[OMX_MAX_POLES];
} omx_medium;

/* TSource (source_mod.f90:7-27), values in a.u. */
typedef struct {
    char   dir;            /* 'x', 'y' or 'z' */
    double j_amp, w0, t0, tau, t_init, t_final, phase;
    double r0[3];
    double radius;
    double chirp;          /* extension, d(omega)/dt in a.u.; 0 reproduces the reference */
} omx_source_desc;

/* Plane-wave soft source (extension; no reference counterpart). */
typedef struct {
    int    comp;           /* 1..3: E component driven */
    int    plane_axis;     /* 1..3 */
    int    plane_index;    /* 1-based cell index along plane_axis */
    double j_amp, w0, t0, tau, t_init, t_final, phase, chirp;
} omx_plane_source_desc;

/* TQ_group (q_group_mod.f90:12-28) with a few-level emitter model behind TQ_sys_base. */
typedef struct {
    int    group_type;     /* OMX_Q_MATERIAL or OMX_Q_SINGLE */
    int    model;          /* OMX_EMITTER_* */
    int    n_systems;
    double density;        /* q_group%density, a.u. */
    double dt;             /* q_group%dt (= n_skip_steps * dt) */
} omx_qgroup_desc;

/* ---- device selection ------------------------------------------------------------------------ */
/* Make `device` current for this host thread; contexts created afterwards live on it.  One
 * process per GPU (the reference's one-rank-per-process model) calls this once at start. */
int omx_select_device(int device);
int omx_device_count(int *count);

/* ---- context (TMxll%init / TMxll%kill) ---------------------------------------------------- */
/* init_{1,2,3}Dgrid: mxll_1D_mod.f90:53, mxll_2D_mod.f90:59, mxll_3D_mod.f90:63.  Computes the
 * CPML tables and den_* arrays exactly as the reference does and zeroes every field. */
int omx_create(const omx_grid_desc *desc, omx_ctx **out);
/* kill_{1,2,3}Dgrid: mxll_3D_mod.f90:435 */
int omx_destroy(omx_ctx *ctx);
const char *omx_last_error(const omx_ctx *ctx);   /* never NULL; ctx may be NULL */
int omx_synchronize(omx_ctx *ctx);

/* CPML tables as computed at create (be,ce[npml]; bh,ch[npml-1]); den arrays per axis. */
int omx_get_cpml_tables(const omx_ctx *ctx, double *be, double *ce, double *bh, double *ch);
int omx_get_den(const omx_ctx *ctx, int axis, double *den_e, double *den_h); /* axis 1..3 */
/* Host-only restatement of the CPML grading (mxll_3D_mod.f90:282-318) for a given npml, dr, dt:
 * be,ce,kappae[npml]; bh,ch,kappah[npml-1].  Needs no device. */
int omx_compute_cpml_tables(int npml, double dr, double dt, double *be, double *ce, double *bh,
                            double *ch, double *kappae, double *kappah);
/* Override the tables, e.g. with the Fortran caller's own arrays (same layout as get). */
int omx_set_cpml_tables(omx_ctx *ctx, const double *be, const double *ce, const double *bh,
                        const double *ch, const double *den_e_x, const double *den_e_y,
                        const double *den_e_z, const double *den_h_x, const double *den_h_y,
                        const double *den_h_z);

/* ---- media (read_init_media_* results; classical_medium_mod.f90:203-769) ------------------- */
/* media[0..n_media-1] describe media 1..n_media.  media_map is the reference's integer array:
 * 3D (nx,ny,nz,3), 2D (nx,ny,3), 1D (nz).  eps_{x,y,z} are the inverse-permittivity arrays
 * (nx,ny,nz) of the reference; pass NULL to derive them from media_map with the reference's
 * rule.  Must precede the first step. */
int omx_set_media(omx_ctx *ctx, int n_media, const omx_medium *media, const int32_t *media_map,
                  const double *eps_x, const double *eps_y, const double *eps_z);

/* Host helpers restating init_classical_medium (classical_medium_mod.f90:46-104). */
int omx_medium_dielectric(double eps_r, omx_medium *m);
int omx_medium_drude(double omegaD, double GammaD, double eps_r, double dt, omx_medium *m);
int omx_medium_dl_library(const char *material, double eps_r, double dt, omx_medium *m);
int omx_medium_dl_custom(double eps_inf, double wp_ev, double gamma_ev, int n_poles,
                         const double *pole_ev, const double *strength, const double *width_ev,
                         double dt, omx_medium *m);   /* extension: A_k = f_k * wp^2 */
/* read_init_media_{1D,2D,3D} voxel rule (file I/O left to the caller): n_vox[m] voxels of
 * medium m+1, coordinates in nm (dims per voxel), media_map out as documented above. */
int omx_media_map_from_voxels(int dimensions, const int grid_Ndims[3], double dr, int n_media,
                              const int *n_vox, const double *vox_nm, int32_t *media_map);

/* ---- time stepping (TMxll%td_propagate_*) --------------------------------------------------- */
/* Every call queues device work and returns.  In the reference's per-step order (omx_step_H,
 * omx_source_interactions, omx_step_E, omx_qgroup_step, omx_detectors_record) the q-group step
 * and the detector record (when every detector samples an E component, or on the fused FP32
 * path) run on the library's side stream next to the next step's first pass; the calls that
 * write E wait for them on the device, and every other entry point orders itself after them. */
int omx_step_H(omx_ctx *ctx);                                  /* td_propagate_H_field */
int omx_step_E(omx_ctx *ctx, double time, double t_skip);      /* td_propagate_E_field */

/* ---- sources (source_mod.f90 / interactions_mod.f90:21-163) -------------------------------- */
int omx_source_add(omx_ctx *ctx, const omx_source_desc *d, int *source_id);  /* init_source */
int omx_plane_source_add(omx_ctx *ctx, const omx_plane_source_desc *d, int *source_id);
/* update_sources + source_interactions for every registered source at `time`. */
int omx_source_interactions(omx_ctx *ctx, double time);

/* ---- emitters (q_group_mod.f90, interactions_mod.f90:167-1220) ------------------------------ */
/* cell: n_systems x dimensions, 1-based local cell indices (q_group%map(:,3:5));
 * params: n_systems x (7 | 9) per the model. */
int omx_qgroup_create(omx_ctx *ctx, const omx_qgroup_desc *d, const int32_t *cell,
                      const double *params, int *group_id);
/* send_E_to_J_ranks + td_propagate_q_group + send_J_to_E_ranks for one group */
int omx_qgroup_step(omx_ctx *ctx, int group_id, int tq_step);
/* dipole, dPt_dt, E (n x 3 each, any may be NULL); rho (n x state) may be NULL */
int omx_qgroup_read(omx_ctx *ctx, int group_id, double *dipole, double *dPt_dt, double *efield,
                    double *rho);
int omx_qgroup_state_size(int model);

/* ---- emitter step without allocation --------------------------------------------------------- */
/* No counterpart in the reference (an addition of this library).
 *
 * For callers that cannot call cudaMalloc -- a host that owns all device memory through its
 * own pool or through Fortran/OpenACC device arrays, and forbids allocation in its time loop
 * because cudaMalloc / cudaFree synchronise the whole device -- this entry point advances a
 * batch of few-level emitters and updates their current arrays entirely in caller-provided
 * device memory, and allocates nothing.  It computes what omx_qgroup_step does
 * after its field gather, from the gathered E samples:
 *   E       n_emitters x 3 device doubles, the E at each emitter (input)
 *   params  n_emitters x 7 | 9 (model), as omx_qgroup_create (input)
 *   rho     n_emitters x omx_qgroup_state_size(model), density matrices (in/out, start at zero)
 *   dipole  n_emitters x 3 (in/out, start at zero)
 *   winner, wk  n_points each: for every current point the index of the emitter that writes it
 *           last (or -1) and its weight (density, or density * kernel weight)
 *   J, J_old, dJ  3 x n_points (component-major): J in/out, J_old and dJ out, for the
 *           components comp_first..comp_last (0-based)
 * All pointers are device pointers; work is queued on `stream` (NULL = default stream).
 * The dP/dt of the emitters, produced by the density-matrix step and consumed by the scatter,
 * lives in a fixed device array of 3 * OMX_NOALLOC_MAX_EMITTERS doubles (1.5 MiB) that every GPU
 * loading the library holds until the process exits.  n_emitters above
 * OMX_NOALLOC_MAX_EMITTERS is rejected with OMX_ERR_ARG.  All calls share that array: calls
 * that overlap on the GPU (other streams, other host threads) race and must be serialised by the
 * caller.  The first call on each device looks the array's device address up (no allocation)
 * and must be made with that device current; make that first call before any stream capture.
 * The array keeps the last call's values; every call overwrites the part it uses before
 * reading it.  Errors are read with omx_last_error(NULL). */
#define OMX_NOALLOC_MAX_EMITTERS 65536
int omx_emitter_step_noalloc(int model, int n_emitters, const double *E, const double *params,
                             double *rho, double *dipole, int n_points, const int *winner,
                             const double *wk, double *J, double *J_old, double *dJ,
                             int comp_first, int comp_last, double dt, void *stream);

/* ---- detectors (write_fields_subs_mod.f90 sampling stencils) ------------------------------- */
/* indx_list: nd x dimensions (TDetector%indx_list, detector_mod.f90:21) */
int omx_detector_add(omx_ctx *ctx, int detector_type, int field, int nd, const int32_t *indx_list,
                     int *detector_id);
int omx_detectors_total_points(const omx_ctx *ctx);
/* sample every detector now into the device record buffer (capacity set here, default 1) */
int omx_detectors_set_capacity(omx_ctx *ctx, int records);
int omx_detectors_record(omx_ctx *ctx, double time);
/* copy out and clear the recorded samples: times[n_rec], values[n_rec x total_points] */
int omx_detectors_drain(omx_ctx *ctx, double *times, double *values, int max_records,
                        int *n_records);
/* Asynchronous drain (the device ring buffer feeding the host writers without a stall): enqueue
 * the copy of every recorded sample into one of OMX_DRAIN_SLOTS pinned slots owned by the
 * library, clear the device records and return at once with a ticket; later steps may be
 * launched right away.  omx_detectors_collect waits for that ticket's copy and hands its records
 * to the caller (times[n_rec], values[n_rec x total_points]; max_records must cover them) and
 * frees the slot.  OMX_ERR_STATE when every slot holds an uncollected ticket.  Behind a
 * one-step omx_run the copies go on the library's side stream and the next one-step call does
 * not wait for them; a host that collects each ticket two steps later never waits either. */
#define OMX_DRAIN_SLOTS 4
int omx_detectors_drain_async(omx_ctx *ctx, long long *ticket);
int omx_detectors_collect(omx_ctx *ctx, long long ticket, double *times, double *values, int max_records,
                          int *n_records);

/* Batched output (the reference opens, appends and closes every file at every print step,
 * write_fields_subs_mod.f90:751-1509): drains every record and writes them in the reference's
 * layout under dir: output_detector_NNNNNNN/point.dat ("time value" lines, appended) and one
 * F_line_/F_plane_/F_volume_PPPPPPPPP.dat per record with a "# Time" header and one line of
 * cell coordinates (nm, the reference's i*dr - int(N/2)*dr) and value per point.  *n_records
 * (may be NULL) receives the number of records written. */
int omx_detectors_write_text(omx_ctx *ctx, const char *dir, int *n_records);
/* Running Fourier transforms of every detector sample, accumulated on the device in FP64 at
 * each record: re/im[k][p] += weight * v_p(t) * (cos, -sin)(omega_k t) (weight: the record
 * interval for a time integral).  Set up after the detectors are added; read resets nothing. */
int omx_detectors_dft_setup(omx_ctx *ctx, int n_freq, const double *omega, double weight);
int omx_detectors_dft_read(omx_ctx *ctx, double *re, double *im);
/* Electromagnetic energy of the grid, FP64 on the device: 0.5 * dr^dims * sum over the interior
 * of eps0 |E|^2 + mu0 |H|^2 (vacuum constants; each component on its own staggered cells). */
int omx_field_energy(omx_ctx *ctx, double *energy);
/* energy_and_dipole.dat of q-group `group` (output_mod.f90:279-331 layout) under
 * dir/output_q_group_NNNN/: a "# Time" header and one line per emitter with its energy
 * Tr(rho H0) in eV and its dipole; append != 0 appends to the file. */
int omx_qgroup_write_text(omx_ctx *ctx, int group, const char *dir, double time, int append);

/* ---- whole driver loop on the device (mxim_mxll.f90:92-132) --------------------------------- */
/* Runs steps tt = tt0 .. tt0+nsteps-1 with the reference's ordering: H, sources, E, q-groups
 * on q-steps, detector records every t_det_print steps (0 disables).  n_skip_steps as in
 * mxim_mxll.f90:73-83.  use_graph != 0 runs the step sequence as a captured CUDA graph; the
 * graph is kept and reused by later calls until a configuration call changes the context. */
int omx_run(omx_ctx *ctx, int tt0, int nsteps, int n_skip_steps, int t_det_print, int use_graph);
/* No counterpart in the reference.  Captures and instantiates the CUDA graphs that
 * omx_run(ctx, tt0, nsteps, n_skip_steps, t_det_print, 1) launches, and sizes the step table
 * and the detector record buffer for it, without running a step (the stepping state, fields
 * and records are unchanged).  A host that calls it before its time loop keeps the capture
 * and instantiation cost out of the loop. */
int omx_run_prepare(omx_ctx *ctx, int tt0, int nsteps, int n_skip_steps, int t_det_print);

/* Kernel form of the FP32 time step (no counterpart in the reference).  Every form meets the same
 * FP32 bar; they differ in rounding, and the form may be changed between steps.
 *   OMX_STEP_DEFAULT      one fused pass per step where eligible (2D TMz; 3D with x and y not
 *                         periodic: the planes staged by TMA, the dispersive cells and a single
 *                         plane source inside the pass), else the two half-step passes
 *   OMX_STEP_TWO_PASS     the two half-step passes everywhere: the arithmetic of batched runs
 *                         (omx_batch_create sets it on its members)
 *   OMX_STEP_SINGLE_PASS  the same as OMX_STEP_DEFAULT */
#define OMX_STEP_DEFAULT 0
#define OMX_STEP_TWO_PASS 1
#define OMX_STEP_SINGLE_PASS 2
int omx_set_step_form(omx_ctx *ctx, int form);

/* Launch-shape autotuner (no counterpart in the reference, whose loops have no launch shape).
 * Times each candidate shape of this grid's field kernels `reps` times and keeps the fastest:
 * the fused FP32 TMz kernel's form (0 register prefetch, 4/5/6/8 bulk-copy ring depth, 14/15/16
 * ring depth 4/5/6 filled by a dedicated copy warp, 24/25 the same with depth 4/5 and two 4-cell
 * chunks per thread, 34/36 register tiles of 4/6 rows, 44/45 depth 4/5 with eight compute warps
 * per block -- 44 is the default), the fused FP32 3D pass's shape (ring depth x 100000 + tile rows
 * x 1000 + planes per block: ring depth 0 (the default, 4) or 2..16 staged planes, rows 8 or 16,
 * 1..128 planes; 8064 is the default) or the planes / rows each thread marches in the unfused
 * kernels.  For a 3D FP32 grid on OMX_STEP_DEFAULT the two half-step passes compete as well
 * (reported as planes per thread, below 1000); when they win, the grid steps with them from then
 * on, as after omx_set_step_form(OMX_STEP_TWO_PASS).  The candidates run on the initial
 * all-zero fields, which every kernel maps to zero, so the simulation state is unchanged: call it
 * after the grid is configured and before the first step or omx_write_field (OMX_ERR_STATE
 * otherwise); configuration calls are closed afterwards, as after a first step.  *choice (may
 * be NULL) receives the chosen shape. */
int omx_autotune(omx_ctx *ctx, int reps, int *choice);
/* Sets the launch shape directly (a value omx_autotune reported, e.g. for a grid of the same shape
 * tuned earlier); no counterpart in the reference.  Every shape of one step form gives the same
 * results bit for bit; on a 3D FP32 grid a shape below 1000 switches to the two half-step passes,
 * whose FP32 results differ from the single pass's by rounding. */
int omx_set_launch_shape(omx_ctx *ctx, int shape);

/* ---- batched multi-grid runs (no counterpart in the reference: it runs one grid per process) -
 * A batch groups n configured 3D contexts of one precision on the current device (for example
 * the instances of a parameter sweep).  omx_batch_run advances all of them together.  When every
 * member steps with the fused FP32 3D pass, each step runs that pass for every grid at once (one
 * launch over all grids' tiles, or for the largest grids the pass split by plane form: their
 * general runs' new H on a second stream beside one launch of their lean runs, then their general
 * runs' new E, the other grids' one launch on that second stream too), one
 * launch per round of the other sources, the per-grid emitter work and one launch for the
 * detectors of every grid.  Otherwise each step runs ONE persistent launch for the H pass of
 * every grid (its blocks walk a list of all grids' tiles), one launch per round of radial sources
 * (round r: source r of every grid), the dispersive cells, ONE launch for the bulk E pass of every
 * grid, the per-grid emitter work and the detectors.  use_graph != 0 captures that step once and
 * replays it.  Every grid computes exactly what omx_run computes for it alone (same arithmetic,
 * same per-grid order).  The contexts stay owned by the caller and must outlive the batch; while
 * omx_batch_run executes, their launches go to the batch's stream. */
typedef struct omx_batch omx_batch;
int omx_batch_create(omx_ctx *const *ctxs, int n, omx_batch **out);
/* The launch shape of the batched passes, each candidate timed `reps` times on the initial zero
 * fields; same preconditions as omx_autotune.  *choice (may be NULL) is the tile depth (z planes
 * per tile: 4, 8, 16 or 32) of the two half-step passes, or for the fused pass
 * s x 1000000 + (ring depth x 100 + tile rows) x 1000 + planes per block: the s largest grids step
 * with the pass split by plane form, the others in one launch over their tiles (s = 0: every grid
 * in that launch); ring depth 0 for the default of 4 planes. */
int omx_batch_autotune(omx_batch *batch, int reps, int *choice);
/* No counterpart in the reference: sets the launch shape of the batched passes, encoded as
 * omx_batch_autotune's choice (a fused shape when every member steps with the fused FP32 pass,
 * else a tile depth); OMX_ERR_ARG for a shape of the other kind or out of range. */
int omx_batch_set_launch_shape(omx_batch *batch, int shape);
int omx_batch_run(omx_batch *batch, int tt0, int nsteps, int n_skip_steps, int t_det_print,
                  int use_graph);
/* No counterpart in the reference: builds the batch's tables and captures the step graphs that
 * omx_batch_run(batch, tt0, nsteps, ..., 1) launches, without running a step. */
int omx_batch_run_prepare(omx_batch *batch, int tt0, int nsteps, int n_skip_steps, int t_det_print);
long long omx_batch_launch_count(const omx_batch *batch);   /* kernels launched by the batch */
/* omx_batch_run returns once the work is queued; this waits for it (and reports kernel errors). */
int omx_batch_synchronize(omx_batch *batch);
int omx_batch_destroy(omx_batch *batch);

/* ---- field access (debug / parity) ---------------------------------------------------------- */
/* Copies a field over the reference's bounds (e.g. 3D Ex(0:nx,1:ny+1,1:nz+1)) to/from host
 * FP64.  The E ghost planes n+1 of periodic axes are closed by index remapping on the device and
 * read back as zero; the H ghost planes 0 of periodic axes hold the wrapped values, as in the
 * reference after its E-step wraps. */
int omx_field_bounds(const omx_ctx *ctx, int field, int lo[3], int hi[3]);
int omx_read_field(omx_ctx *ctx, int field, double *host);
int omx_write_field(omx_ctx *ctx, int field, const double *host);

/* ---- measurement ------------------------------------------------------------------------------ */
/* Per-kernel timing with CUDA events on the context's stream: enable, run, then query the
 * accumulated milliseconds and launch count of a kernel class (0 = H update, 1 = E update,
 * 2 = emitters, 3 = sources, 4 = detectors). */
int omx_profile_enable(omx_ctx *ctx, int on);
int omx_profile_query(omx_ctx *ctx, int kernel_class, double *total_ms, long long *launches);
/* algorithmic bytes moved by one launch of a kernel class in the current configuration */
int omx_algorithmic_bytes(const omx_ctx *ctx, int kernel_class, double *bytes);
/* number of library kernel launches issued since creation */
long long omx_launch_count(const omx_ctx *ctx);
/* events around a region on the context stream */
int omx_timer_start(omx_ctx *ctx);
int omx_timer_stop(omx_ctx *ctx, float *ms);
/* flush L2 by writing a scratch buffer larger than L2 on the context stream */
int omx_flush_l2(omx_ctx *ctx);

/* ---- learned emitter closure: building blocks ----------------------------------------------- */
/* BF16 GEMM on the tensor cores (tcgen05 MMA, TMA-staged operands, FP32 accumulation in tensor
 * memory), the building block of the closure's training and inference; exposed on host arrays for
 * validation.  D[M x N] = act(alpha * A[M x K] * B[N x K]^T + bias[N]) with A, B raw BF16 bits,
 * row-major, K contiguous (K a multiple of 8); bias may be NULL; act: 0 none, 1 tanh,
 * 2 logistic sigmoid, 3 relu.  No reference counterpart. */
int omx_tc_gemm_bf16(const uint16_t *A, const uint16_t *B, const float *bias, float *D, int M, int N, int K,
                     float alpha, int act);

/* The closure network (no reference counterpart).  Per emitter and quantum step: a GRU (hidden
 * 128) over the last 32 samples of the local field on the emitter's dipole axis, a tanh MLP
 * (3 layers of 256) and a linear read-out of the dipole on that axis; BF16 tensor-core GEMMs
 * with FP32 accumulation, FP32 state and master weights, Adam.  Sequences are e[B][T + 31]
 * (scaled field samples, step t sees e[b][t .. t+31]) and y / target[T][B] (scaled dipoles);
 * B must be a multiple of 8.  Parameters are a flat FP32 vector of omx_closure_n_params()
 * values in the order Wg[512 x 160], bg[512], W1[256 x 128], b1, W2[256 x 256], b2, W3, b3,
 * w4[256], b4[1]; e_scale / d_scale record the field and dipole units of the scaled data. */
typedef struct omx_closure omx_closure;
int omx_closure_create(omx_closure **out);
int omx_closure_destroy(omx_closure *cl);
long long omx_closure_n_params(void);
int omx_closure_set_params(omx_closure *cl, const float *params, double e_scale, double d_scale);
int omx_closure_get_params(omx_closure *cl, float *params, double *e_scale, double *d_scale);
int omx_closure_forward(omx_closure *cl, const float *e, int B, int T, float *y);
/* loss = mean over t >= skip of (y - target)^2 and its gradient (no update) */
int omx_closure_gradient(omx_closure *cl, const float *e, const float *target, int B, int T, int skip,
                         float *grad, double *loss);
/* one Adam step (beta 0.9 / 0.999) on that loss; *loss is the loss before the step */
int omx_closure_train_step(omx_closure *cl, const float *e, const float *target, int B, int T, int skip,
                           float lr, double *loss);
/* Training data from the plain propagator (the q-groups' FP64 RK4 emitter model): n emitters
 * (params[n][7 or 9] as in omx_qgroup_create) start in the ground state and are driven by
 * E(t_s) = amp * sum_k c_k cos(w_k t_s + phi_k), t_s = s * dt, with drive[n][1 + 3K] =
 * (amp, c_1, w_1, phi_1, ...); outputs e[n][T] = E(t_s) / e_scale and d[n][T] = the dipole
 * along the emitter axis after step s, / d_scale. */
int omx_closure_trajectories(int model, int n, int T, int K, double dt, const double *params,
                             const double *drive, double e_scale, double d_scale, float *e, float *d);
/* Deploy a trained closure on q-group `group` (before the first step; the closure must outlive
 * the context).  Each quantum step, the network maps every emitter's last 32 field samples on its
 * dipole axis and its GRU state to its dipole (dP/dt and the current scatter as for the plain
 * model).  A spot-check subset (check_fraction of the group, spread evenly) is propagated by the
 * plain FP64 model with the same fields; every check_every steps the error max|network - plain|
 * / max|plain| over the subset and those steps is compared with tol.  Above tol the plain
 * propagator takes over for the rest of the run: the subset keeps its exact state, every other
 * emitter restarts from the ground state replayed through its stored 32-sample window (earlier
 * history is lost).  All decisions are taken on the device, inside captured graphs too. */
int omx_qgroup_attach_closure(omx_ctx *ctx, int group, omx_closure *cl, double check_fraction, double tol,
                              int check_every);
/* last completed check's error, whether the plain propagator took over and at which closure step
 * (-1 if not), and the number of checks so far */
int omx_qgroup_closure_status(omx_ctx *ctx, int group, double *last_error, int *fallback,
                              int *fallback_step, int *checks);

/* ---- frequency-domain operator of the inverse-design program ---------------------------------
 * src/freq_domain_inverse_design/operator_mod.f90: init_operator (:41-232), apply_operator_1D
 * (:293-361), _2D (:364-514), _3D (:518-710); bicgstab_mod.f90:76-243: BICGStab_L.  FP64, the
 * program's units (c0 = eps0 = mu0 = 1).  Vectors are complex components -- 3D and 2D: pl_x,
 * pl_y, pl_z, mi_x, mi_y, mi_z; 1D: pl_x, pl_y, mi_x, mi_y -- each over [1-g, n+g] along every
 * active axis (g = n_der ghost cells), x fastest, as interleaved (re, im) doubles:
 * omx_fd_vector_length complex values.  eps_r: the grid's nx*ny*nz complex values, x fastest
 * (ny = nz = 1 below 3D).  boundaries (per active axis): 1 close, 2 periodic (the reference's
 * ghost copies, including the 3D y-axis copies of mi_x into the low ghosts only and mi_y into the
 * high ghosts only), 3 PML (n_pml cells). */
typedef struct omx_fdop omx_fdop;
int omx_fd_create(int dimensions, const int grid_Ndims[3], int n_pml, int n_der, const int boundaries[3], double dr,
                  double w0, const double *eps_r, omx_fdop **out);
int omx_fd_destroy(omx_fdop *op);
/* replace eps_r (the design's permittivity after an optimisation step; the reference passes its
 * TMedium_eps_r to every apply_operator / BICGStab_L call) */
int omx_fd_set_eps(omx_fdop *op, const double *eps_r);
long long omx_fd_vector_length(const omx_fdop *op);
/* Af = A f (transpose != 0: the adjoint form, C1 negated); f's periodic ghosts are refreshed */
int omx_fd_apply(omx_fdop *op, const double *f, double *Af, int transpose);
/* BiCGStab(L) for A f = j from the guess in f (solution returned in f); converged, the final
 * relative residual |r| / |j| and the outer iteration count are returned */
int omx_fd_solve(omx_fdop *op, const double *j, double *f, int transpose, double tol, int n_max, int L,
                 int *converged, double *abs_err, int *iterations);
/* measurement: mean time of reps applications on device-resident vectors (CUDA events) */
int omx_fd_time_apply(omx_fdop *op, int reps, double *ms_per_apply);

#ifdef __cplusplus
}
#endif
#endif
