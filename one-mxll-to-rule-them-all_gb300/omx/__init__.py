"""Python mirror of OMxRTA's time-domain plugin interface over the GB300 C-ABI library.

`TMxll` follows the reference's TMxll type (src/FDTD/mxll_base_mod.f90:7-69): `init` is the
constructor, `kill`, `td_propagate_H_field`, `td_propagate_E_field`; the free routines called by
the reference's time loop (src/FDTD/mxim_mxll.f90:92-132) are methods with the reference's
names: `source_interactions`, `send_E_to_J_ranks` + `td_propagate_q_group` +
`send_J_to_E_ranks` (one batched call per q-group), and `write_detectors_outputs` (sampling
only; the text formatting stays with the caller).  Arrays use the reference's Fortran index
order and bounds.  Every call raises OMXError on a non-zero status, as the reference stops.
"""
import ctypes as C

import numpy as np

from . import _capi as A
from ._capi import (CLOSE, CPML, DIELECTRIC, DL, DRUDE, EX, EY, EZ, FIELDS, HX, HY, HZ, KC_DET, KC_E,
                    KC_EMIT, KC_H, KC_SRC, LINE_X, LINE_Y, LINE_Z, NONE_MEDIUM, PERIODIC, PLANE_XY,
                    PLANE_YZ, PLANE_ZX, POINT, PREC_FP32, PREC_FP64, Q_MATERIAL, Q_SINGLE, STEP_DEFAULT,
                    STEP_SINGLE_PASS, STEP_TWO_PASS, TEZ, THREE_LEVEL, TMZ, TWO_LEVEL, VOLUME, OMXError, lib)
from .units import UNITS

__all__ = ["TMxll", "Medium", "OMXError", "lib", "UNITS", "medium_dielectric", "medium_drude",
           "medium_dl_library", "medium_dl_custom", "media_map_from_voxels"]


def _medium_call(fn, *args):
    m = A.Medium()
    A.check(fn(*args, C.byref(m)))
    return m


def medium_dielectric(eps_r):
    return _medium_call(lib().omx_medium_dielectric, float(eps_r))


def medium_drude(omegaD, GammaD, eps_r, dt):
    """init_classical_medium 'drude' (classical_medium_mod.f90:64-74); omegaD, GammaD in a.u."""
    return _medium_call(lib().omx_medium_drude, float(omegaD), float(GammaD), float(eps_r), float(dt))


def medium_dl_library(material, eps_r, dt):
    """init_classical_medium 'drude-lorentz' with the Ag/Al/Au library (:76-100, :125-199)."""
    return _medium_call(lib().omx_medium_dl_library, material.encode(), float(eps_r), float(dt))


def medium_dl_custom(eps_inf, wp_ev, gamma_ev, poles_ev, strengths, widths_ev, dt):
    """Extension: user-defined Drude-Lorentz poles with the reference's ADE arithmetic."""
    p = A.as_f64(poles_ev)
    s = A.as_f64(strengths)
    w = A.as_f64(widths_ev)
    return _medium_call(lib().omx_medium_dl_custom, float(eps_inf), float(wp_ev), float(gamma_ev), len(p),
                        A.dptr(p), A.dptr(s), A.dptr(w), float(dt))


Medium = A.Medium


def media_map_from_voxels(dimensions, grid_Ndims, dr, voxels_per_medium):
    """read_init_media_{1D,2D,3D} voxel rule.  voxels_per_medium: list of (n, dims) arrays in nm.
    Returns media_map in Fortran shape ((nx,ny,nz,3) / (nx,ny,3) / (nz,))."""
    dims = int(dimensions)
    n = [int(v) for v in grid_Ndims] + [1] * (3 - len(grid_Ndims))
    counts = np.array([len(v) for v in voxels_per_medium], dtype=np.int32)
    vox = (np.concatenate([np.asarray(v, dtype=np.float64).reshape(-1, dims) for v in voxels_per_medium])
           if len(voxels_per_medium) and counts.sum() else np.zeros((0, dims)))
    vox = np.ascontiguousarray(vox.reshape(-1))
    if dims == 1:
        shape = (n[0],)
    elif dims == 2:
        shape = (n[0], n[1], 3)
    else:
        shape = (n[0], n[1], n[2], 3)
    out = np.zeros(int(np.prod(shape)), dtype=np.int32)
    nd = (C.c_int * 3)(*n)
    A.check(lib().omx_media_map_from_voxels(dims, nd, float(dr), len(counts),
                                            counts.ctypes.data_as(A._PI), A.dptr(vox), A.iptr(out)))
    return out.reshape(shape, order="F")


class QGroup:
    def __init__(self, mxll, gid, desc, n):
        self.mxll, self.gid, self.desc, self.n_systems = mxll, gid, desc, n

    def read(self):
        n = self.n_systems
        dip = np.zeros((n, 3))
        dpdt = np.zeros((n, 3))
        ef = np.zeros((n, 3))
        rho = np.zeros((n, lib().omx_qgroup_state_size(self.desc.model)))
        A.check(lib().omx_qgroup_read(self.mxll._ctx, self.gid, A.dptr(dip), A.dptr(dpdt), A.dptr(ef),
                                      A.dptr(rho)), self.mxll._ctx)
        return {"dipole": dip, "dPt_dt": dpdt, "E": ef, "rho": rho}

    def attach_closure(self, closure, check_fraction=0.01, tol=1e-3, check_every=16):
        """Run this group's emitters through a trained closure, with a spot-check subset on the
        plain propagator that takes over above `tol` (omx_qgroup_attach_closure)."""
        A.check(lib().omx_qgroup_attach_closure(self.mxll._ctx, self.gid, closure._c, float(check_fraction),
                                                float(tol), int(check_every)), self.mxll._ctx)
        self._closure = closure                  # the closure must outlive the context

    def write_text(self, directory, time, append=False):
        """energy_and_dipole.dat of this group in the reference's layout."""
        A.check(lib().omx_qgroup_write_text(self.mxll._ctx, self.gid, str(directory).encode(), float(time),
                                            1 if append else 0), self.mxll._ctx)

    def closure_status(self):
        err, fb, step, checks = C.c_double(), C.c_int(), C.c_int(), C.c_int()
        A.check(lib().omx_qgroup_closure_status(self.mxll._ctx, self.gid, C.byref(err), C.byref(fb), C.byref(step),
                                                C.byref(checks)), self.mxll._ctx)
        return {"last_error": err.value, "fallback": bool(fb.value), "fallback_step": step.value,
                "checks": checks.value}


class TMxll:
    """GPU drop-in for TMxll_1D/2D/3D (init_{1,2,3}Dgrid ... td_propagate_E_field)."""

    def __init__(self, dimensions, grid_Ndims, npml, boundaries, dt, dr, mode=TMZ, precision="fp64"):
        d = A.GridDesc()
        d.dimensions = int(dimensions)
        g = list(grid_Ndims) + [1] * (3 - len(grid_Ndims))
        d.grid_Ndims = (C.c_int * 3)(*[int(v) for v in g])
        d.npml = int(npml)
        b = list(boundaries) + [CLOSE] * (3 - len(boundaries))
        d.boundaries = (C.c_int * 3)(*[int(v) for v in b])
        d.mode = int(mode)
        d.precision = PREC_FP32 if precision in ("fp32", PREC_FP32) else PREC_FP64
        d.dt = float(dt)
        d.dr = float(dr)
        self.desc = d
        self.dimensions = int(dimensions)
        self.grid_Ndims = tuple(int(v) for v in g[:self.dimensions])
        self.mode = int(mode)
        self.dt, self.dr = float(dt), float(dr)
        self._ctx = C.c_void_p()
        A.check(lib().omx_create(C.byref(d), C.byref(self._ctx)))
        self.groups = []
        self.sources = []
        self.detectors = []
        self.time = 0.0
        self.t_skip = 0.0

    # -- lifecycle ---------------------------------------------------------------------------
    def kill(self):
        if self._ctx:
            lib().omx_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.kill()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.kill()

    def _chk(self, rc):
        A.check(rc, self._ctx)

    def synchronize(self):
        self._chk(lib().omx_synchronize(self._ctx))

    # -- set-up -------------------------------------------------------------------------------
    def cpml_tables(self):
        npml = self.desc.npml
        be, ce = np.zeros(npml), np.zeros(npml)
        bh, ch = np.zeros(npml - 1), np.zeros(npml - 1)
        self._chk(lib().omx_get_cpml_tables(self._ctx, A.dptr(be), A.dptr(ce), A.dptr(bh), A.dptr(ch)))
        return be, ce, bh, ch

    def den(self, axis):
        n = self.grid_Ndims[axis - 1] if axis <= self.dimensions else 1
        de, dh = np.zeros(n), np.zeros(n)
        self._chk(lib().omx_get_den(self._ctx, int(axis), A.dptr(de), A.dptr(dh)))
        return de, dh

    def set_media(self, media, media_map, eps=None):
        arr = (A.Medium * max(1, len(media)))(*media) if media else (A.Medium * 1)()
        mm = A.fortran_flat_i32(media_map) if media_map is not None else None
        e = [None, None, None]
        if eps is not None:
            e = [A.fortran_flat_f64(x) if x is not None else None for x in eps]
        self._chk(lib().omx_set_media(self._ctx, len(media), arr, A.iptr(mm), A.dptr(e[0]), A.dptr(e[1]),
                                      A.dptr(e[2])))

    def add_source(self, direction, j_amp, w0, t0, tau, r0, radius, t_init, t_final, phase=0.0, chirp=0.0):
        """init_source (source_mod.f90:37-102); values in a.u."""
        s = A.SourceDesc()
        s.dir = direction.encode()
        s.j_amp, s.w0, s.t0, s.tau = j_amp, w0, t0, tau
        s.t_init, s.t_final, s.phase = t_init, t_final, phase
        s.r0 = (C.c_double * 3)(*[float(v) for v in list(r0) + [0.0] * (3 - len(r0))])
        s.radius = radius
        s.chirp = chirp
        sid = C.c_int()
        self._chk(lib().omx_source_add(self._ctx, C.byref(s), C.byref(sid)))
        self.sources.append(s)
        return sid.value

    def add_plane_source(self, comp, plane_axis, plane_index, j_amp, w0, t0, tau, t_init, t_final, phase=0.0,
                         chirp=0.0):
        s = A.PlaneSourceDesc()
        s.comp, s.plane_axis, s.plane_index = int(comp), int(plane_axis), int(plane_index)
        s.j_amp, s.w0, s.t0, s.tau, s.t_init, s.t_final, s.phase, s.chirp = (
            j_amp, w0, t0, tau, t_init, t_final, phase, chirp)
        sid = C.c_int()
        self._chk(lib().omx_plane_source_add(self._ctx, C.byref(s), C.byref(sid)))
        self.sources.append(s)
        return sid.value

    def add_q_group(self, group_type, model, cells, params, density, dt):
        """init_q_group + init_all_q_systems for a few-level emitter model (batched)."""
        cells = np.ascontiguousarray(np.asarray(cells, dtype=np.int32).reshape(-1, self.dimensions))
        params = np.ascontiguousarray(np.asarray(params, dtype=np.float64))
        n = cells.shape[0]
        d = A.QGroupDesc()
        d.group_type, d.model, d.n_systems, d.density, d.dt = int(group_type), int(model), n, density, dt
        gid = C.c_int()
        self._chk(lib().omx_qgroup_create(self._ctx, C.byref(d), A.iptr(cells), A.dptr(params), C.byref(gid)))
        g = QGroup(self, gid.value, d, n)
        self.groups.append(g)
        return g

    def add_detector(self, detector_type, field, indx_list):
        """TDetector with its index list (detector_mod.f90:21), shape (nd, dimensions)."""
        idx = np.asarray(indx_list, dtype=np.int32).reshape(-1, self.dimensions)
        flat = np.ascontiguousarray(idx.reshape(-1, order="F"))
        f = FIELDS[field] if isinstance(field, str) else int(field)
        did = C.c_int()
        self._chk(lib().omx_detector_add(self._ctx, int(detector_type), f, idx.shape[0], A.iptr(flat),
                                         C.byref(did)))
        self.detectors.append((detector_type, f, idx.shape[0]))
        return did.value

    # -- the reference's per-step calls -------------------------------------------------------
    def td_propagate_H_field(self):
        self._chk(lib().omx_step_H(self._ctx))

    def td_propagate_E_field(self, time=None, t_skip=None):
        t = self.time if time is None else time
        ts = self.t_skip if t_skip is None else t_skip
        self._chk(lib().omx_step_E(self._ctx, float(t), float(ts)))

    def source_interactions(self, time):
        """update_sources + source_interactions (source_mod.f90:234, interactions_mod.f90:21)."""
        self._chk(lib().omx_source_interactions(self._ctx, float(time)))

    def q_group_step(self, group, tq_step=1):
        """send_E_to_J_ranks + td_propagate_q_group + send_J_to_E_ranks for one group."""
        self._chk(lib().omx_qgroup_step(self._ctx, group.gid, int(tq_step)))

    def write_detectors_outputs(self, time):
        """Sample every detector now into the device record buffer."""
        self._chk(lib().omx_detectors_record(self._ctx, float(time)))

    def drain_detectors(self, max_records=1 << 20):
        npts = lib().omx_detectors_total_points(self._ctx)
        nrec = C.c_int()
        # query count by draining into large enough buffers
        times = np.zeros(max_records)
        vals = np.zeros((max_records, max(npts, 1)))
        self._chk(lib().omx_detectors_drain(self._ctx, A.dptr(times), A.dptr(vals), max_records, C.byref(nrec)))
        n = nrec.value
        return times[:n].copy(), vals[:n, :npts].copy()

    def set_step_form(self, form):
        """Kernel form of the FP32 step: STEP_DEFAULT, STEP_TWO_PASS (the batch arithmetic) or
        STEP_SINGLE_PASS."""
        self._chk(lib().omx_set_step_form(self._ctx, int(form)))

    def drain_async(self):
        """Enqueue the copy of the recorded samples into a pinned slot; returns a ticket."""
        t = C.c_longlong()
        self._chk(lib().omx_detectors_drain_async(self._ctx, C.byref(t)))
        return t.value

    def collect(self, ticket, max_records=64):
        """Wait for a ticket's copy; returns (times, values) like drain_detectors."""
        npts = lib().omx_detectors_total_points(self._ctx)
        nrec = C.c_int()
        times = np.zeros(max_records)
        vals = np.zeros((max_records, max(npts, 1)))
        self._chk(lib().omx_detectors_collect(self._ctx, int(ticket), A.dptr(times), A.dptr(vals), int(max_records),
                                              C.byref(nrec)))
        n = nrec.value
        return times[:n].copy(), vals[:n, :npts].copy()

    def run(self, tt0, nsteps, n_skip_steps=1, t_det_print=0, use_graph=True):
        """The reference's time loop (mxim_mxll.f90:92-132) on the device."""
        self._chk(lib().omx_run(self._ctx, int(tt0), int(nsteps), int(n_skip_steps), int(t_det_print),
                                1 if use_graph else 0))

    def prepare_run(self, tt0, nsteps, n_skip_steps=1, t_det_print=0):
        """Capture the step graphs `run(tt0, nsteps, ...)` launches, without running a step."""
        self._chk(lib().omx_run_prepare(self._ctx, int(tt0), int(nsteps), int(n_skip_steps), int(t_det_print)))

    def write_detectors_text(self, directory):
        """Drain the records into the reference's detector file layout; returns the count."""
        n = C.c_int()
        self._chk(lib().omx_detectors_write_text(self._ctx, str(directory).encode(), C.byref(n)))
        return n.value

    def dft_setup(self, omega, weight):
        om = np.ascontiguousarray(omega, np.float64)
        self._dft_n = om.size
        self._chk(lib().omx_detectors_dft_setup(self._ctx, om.size, A.dptr(om), float(weight)))

    def dft_read(self):
        npts = lib().omx_detectors_total_points(self._ctx)
        re = np.zeros((self._dft_n, npts))
        im = np.zeros((self._dft_n, npts))
        self._chk(lib().omx_detectors_dft_read(self._ctx, A.dptr(re), A.dptr(im)))
        return re + 1j * im

    def field_energy(self):
        e = C.c_double()
        self._chk(lib().omx_field_energy(self._ctx, C.byref(e)))
        return e.value

    def autotune(self, reps=20):
        """Pick this grid's kernel launch shape by timing the candidates on the initial zero
        fields (before the first step); returns the chosen shape."""
        choice = C.c_int()
        self._chk(lib().omx_autotune(self._ctx, int(reps), C.byref(choice)))
        return choice.value

    def set_launch_shape(self, shape):
        """Use a launch shape omx_autotune reported (results are the same bit for bit)."""
        self._chk(lib().omx_set_launch_shape(self._ctx, int(shape)))

    # -- field access ----------------------------------------------------------------------------
    def field_bounds(self, field):
        lo = (C.c_int * 3)()
        hi = (C.c_int * 3)()
        f = FIELDS[field] if isinstance(field, str) else int(field)
        self._chk(lib().omx_field_bounds(self._ctx, f, lo, hi))
        return list(lo), list(hi)

    def read_field(self, field):
        """Field over the reference's bounds as a Fortran-ordered array (lo-based indices)."""
        lo, hi = self.field_bounds(field)
        shape = tuple(hi[a] - lo[a] + 1 for a in range(3))
        out = np.zeros(int(np.prod(shape)))
        f = FIELDS[field] if isinstance(field, str) else int(field)
        self._chk(lib().omx_read_field(self._ctx, f, A.dptr(out)))
        return out.reshape(shape, order="F")

    def write_field(self, field, values):
        f = FIELDS[field] if isinstance(field, str) else int(field)
        flat = A.fortran_flat_f64(values)
        self._chk(lib().omx_write_field(self._ctx, f, A.dptr(flat)))

    # -- measurement ----------------------------------------------------------------------------
    def profile(self, on=True):
        self._chk(lib().omx_profile_enable(self._ctx, 1 if on else 0))

    def profile_query(self, kernel_class):
        ms = C.c_double()
        n = C.c_longlong()
        self._chk(lib().omx_profile_query(self._ctx, int(kernel_class), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def algorithmic_bytes(self, kernel_class):
        b = C.c_double()
        self._chk(lib().omx_algorithmic_bytes(self._ctx, int(kernel_class), C.byref(b)))
        return b.value

    def launch_count(self):
        return int(lib().omx_launch_count(self._ctx))

    def timer_start(self):
        self._chk(lib().omx_timer_start(self._ctx))

    def timer_stop(self):
        ms = C.c_float()
        self._chk(lib().omx_timer_stop(self._ctx, C.byref(ms)))
        return ms.value

    def flush_l2(self):
        self._chk(lib().omx_flush_l2(self._ctx))


def compute_cpml_tables(npml, dr, dt):
    """Host-only CPML grading tables: be, ce, bh, ch, kappae, kappah."""
    be, ce, ke = np.zeros(npml), np.zeros(npml), np.zeros(npml)
    bh, ch, kh = np.zeros(npml - 1), np.zeros(npml - 1), np.zeros(npml - 1)
    A.check(lib().omx_compute_cpml_tables(int(npml), float(dr), float(dt), A.dptr(be), A.dptr(ce), A.dptr(bh),
                                          A.dptr(ch), A.dptr(ke), A.dptr(kh)))
    return be, ce, bh, ch, ke, kh


def select_device(device):
    """Make a CUDA device current for the contexts this process creates afterwards."""
    A.check(lib().omx_select_device(int(device)))


def device_count():
    n = C.c_int()
    A.check(lib().omx_device_count(C.byref(n)))
    return n.value


class Batch:
    """Several configured 3D grids of one precision advanced together (omx_batch_*): one
    persistent launch per pass over all grids' tiles, the step captured in a CUDA graph.  Each
    grid computes exactly what its own `run` would."""

    def __init__(self, grids):
        self.grids = list(grids)
        arr = (C.c_void_p * len(self.grids))(*[g._ctx.value for g in self.grids])
        self._b = C.c_void_p()
        A.check(lib().omx_batch_create(arr, len(self.grids), C.byref(self._b)))

    def autotune(self, reps=10):
        """Launch shape of the batched passes, timed on the zero initial fields; returns it
        (encoded as omx_batch_autotune describes)."""
        choice = C.c_int()
        A.check(lib().omx_batch_autotune(self._b, int(reps), C.byref(choice)))
        return choice.value

    def set_launch_shape(self, shape):
        """Launch shape of the batched passes, encoded as autotune returns it."""
        A.check(lib().omx_batch_set_launch_shape(self._b, int(shape)))

    def drain_async(self):
        """Enqueue the copy of the recorded samples into a pinned slot; returns a ticket."""
        t = C.c_longlong()
        self._chk(lib().omx_detectors_drain_async(self._ctx, C.byref(t)))
        return t.value

    def collect(self, ticket, max_records=64):
        """Wait for a ticket's copy; returns (times, values) like drain_detectors."""
        npts = lib().omx_detectors_total_points(self._ctx)
        nrec = C.c_int()
        times = np.zeros(max_records)
        vals = np.zeros((max_records, max(npts, 1)))
        self._chk(lib().omx_detectors_collect(self._ctx, int(ticket), A.dptr(times), A.dptr(vals), int(max_records),
                                              C.byref(nrec)))
        n = nrec.value
        return times[:n].copy(), vals[:n, :npts].copy()

    def run(self, tt0, nsteps, n_skip_steps=1, t_det_print=0, use_graph=True):
        A.check(lib().omx_batch_run(self._b, int(tt0), int(nsteps), int(n_skip_steps), int(t_det_print),
                                    1 if use_graph else 0))

    def prepare_run(self, tt0, nsteps, n_skip_steps=1, t_det_print=0):
        """Build the tables and capture the step graphs `run(tt0, nsteps, ...)` launches."""
        A.check(lib().omx_batch_run_prepare(self._b, int(tt0), int(nsteps), int(n_skip_steps), int(t_det_print)))

    def launch_count(self):
        return int(lib().omx_batch_launch_count(self._b))

    def synchronize(self):
        A.check(lib().omx_batch_synchronize(self._b))

    def kill(self):
        if self._b:
            lib().omx_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __del__(self):
        try:
            self.kill()
        except Exception:
            pass


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def closure_trajectories(model, params, drive, T, dt, e_scale, d_scale):
    """Plain-propagator training trajectories (omx_closure_trajectories): returns e, d [n][T]."""
    params = np.ascontiguousarray(params, np.float64)
    drive = np.ascontiguousarray(drive, np.float64)
    n = params.shape[0]
    K = (drive.shape[1] - 1) // 3
    e = np.zeros((n, T), np.float32)
    d = np.zeros((n, T), np.float32)
    A.check(lib().omx_closure_trajectories(int(model), n, int(T), K, float(dt), A.dptr(params), A.dptr(drive),
                                           float(e_scale), float(d_scale), _fptr(e), _fptr(d)))
    return e, d


class Closure:
    """The learned emitter closure (omx_closure_*): GRU(128) + MLP(3 x 256) trained and run on the
    tensor cores in BF16 with FP32 accumulation."""

    def __init__(self, params=None, e_scale=1.0, d_scale=1.0):
        self._c = C.c_void_p()
        A.check(lib().omx_closure_create(C.byref(self._c)))
        self.n_params = int(lib().omx_closure_n_params())
        if params is not None:
            self.set_params(params, e_scale, d_scale)

    def set_params(self, params, e_scale=1.0, d_scale=1.0):
        p = np.ascontiguousarray(params, np.float32)
        assert p.size == self.n_params
        A.check(lib().omx_closure_set_params(self._c, _fptr(p), float(e_scale), float(d_scale)))

    def get_params(self):
        p = np.zeros(self.n_params, np.float32)
        es, ds = C.c_double(), C.c_double()
        A.check(lib().omx_closure_get_params(self._c, _fptr(p), C.byref(es), C.byref(ds)))
        return p, es.value, ds.value

    def forward(self, e, T):
        e = np.ascontiguousarray(e, np.float32)
        B = e.shape[0]
        y = np.zeros((T, B), np.float32)
        A.check(lib().omx_closure_forward(self._c, _fptr(e), B, int(T), _fptr(y)))
        return y

    def gradient(self, e, target, skip=0):
        e = np.ascontiguousarray(e, np.float32)
        t = np.ascontiguousarray(target, np.float32)
        g = np.zeros(self.n_params, np.float32)
        loss = C.c_double()
        A.check(lib().omx_closure_gradient(self._c, _fptr(e), _fptr(t), e.shape[0], t.shape[0], int(skip), _fptr(g),
                                           C.byref(loss)))
        return loss.value, g

    def train_step(self, e, target, lr, skip=0):
        e = np.ascontiguousarray(e, np.float32)
        t = np.ascontiguousarray(target, np.float32)
        loss = C.c_double()
        A.check(lib().omx_closure_train_step(self._c, _fptr(e), _fptr(t), e.shape[0], t.shape[0], int(skip),
                                             float(lr), C.byref(loss)))
        return loss.value

    def kill(self):
        if self._c:
            lib().omx_closure_destroy(self._c)
            self._c = C.c_void_p()

    def __del__(self):
        try:
            self.kill()
        except Exception:
            pass


class FDOperator:
    """The frequency-domain operator of the inverse-design program and its BiCGStab(L) solver
    (omx_fd_*) on a 1D, 2D or 3D grid n.  Vectors: complex arrays [6][nz+2g][ny+2g][nx+2g] (3D),
    [6][ny+2g][nx+2g] (2D), [4][nx+2g] (1D), g = n_der; eps of shape n."""

    def __init__(self, n, n_pml, n_der, boundaries, dr, w0, eps):
        self.n, self.g = tuple(int(v) for v in n), int(n_der)
        dims = len(self.n)
        e = np.ascontiguousarray(np.asarray(eps, np.complex128).reshape(self.n).transpose())
        nn = (C.c_int * 3)(*(list(self.n) + [1] * (3 - dims)))
        bb = (C.c_int * 3)(*([int(b) for b in boundaries] + [1] * (3 - len(boundaries))))
        self._op = C.c_void_p()
        A.check(lib().omx_fd_create(dims, nn, int(n_pml), int(n_der), bb, float(dr), float(w0),
                                    e.view(np.float64).ctypes.data_as(A._PD), C.byref(self._op)))

    def shape(self):
        g = self.g
        pad = tuple(v + 2 * g for v in reversed(self.n))
        return ((4,) if len(self.n) == 1 else (6,)) + pad

    def zeros(self):
        return np.zeros(self.shape(), np.complex128)

    def apply(self, f, transpose=False):
        f = np.ascontiguousarray(f, np.complex128)
        out = self.zeros()
        A.check(lib().omx_fd_apply(self._op, f.view(np.float64).ctypes.data_as(A._PD),
                                   out.view(np.float64).ctypes.data_as(A._PD), 1 if transpose else 0))
        return out

    def solve(self, j, f0, tol, n_max, L, transpose=False):
        j = np.ascontiguousarray(j, np.complex128)
        f = np.ascontiguousarray(f0, np.complex128).copy()
        conv, err, it = C.c_int(), C.c_double(), C.c_int()
        A.check(lib().omx_fd_solve(self._op, j.view(np.float64).ctypes.data_as(A._PD),
                                   f.view(np.float64).ctypes.data_as(A._PD), 1 if transpose else 0, float(tol),
                                   int(n_max), int(L), C.byref(conv), C.byref(err), C.byref(it)))
        return f, bool(conv.value), err.value, it.value

    def set_eps(self, eps):
        e = np.ascontiguousarray(np.asarray(eps, np.complex128).reshape(self.n).transpose())
        A.check(lib().omx_fd_set_eps(self._op, e.view(np.float64).ctypes.data_as(A._PD)))

    def time_apply(self, reps=20):
        ms = C.c_double()
        A.check(lib().omx_fd_time_apply(self._op, int(reps), C.byref(ms)))
        return ms.value

    def kill(self):
        if self._op:
            lib().omx_fd_destroy(self._op)
            self._op = C.c_void_p()

    def __del__(self):
        try:
            self.kill()
        except Exception:
            pass
