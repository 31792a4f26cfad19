"""ctypes wrapper of the CPU FP64 oracle (oracle/omx_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg, never by the product path.  Parity against the reference itself is unpinned (no
Fortran compiler, no reference tests or golden vectors); see omx_oracle.h.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liborc.so")
MAXP = 8

_lib = None


class OrcMedium(C.Structure):
    _fields_ = [("medium_type", C.c_int), ("n_poles", C.c_int), ("eps_r", C.c_double),
                ("A1", C.c_double), ("A2", C.c_double), ("C1", C.c_double), ("C2", C.c_double),
                ("C3", C.c_double), ("C4", C.c_double),
                ("alpha_k", C.c_double * MAXP), ("beta_k", C.c_double * MAXP),
                ("gamma_k", C.c_double * MAXP), ("B1_k", C.c_double * MAXP), ("B2_k", C.c_double * MAXP),
                ("omegaD", C.c_double), ("GammaD", C.c_double), ("omegaP", C.c_double),
                ("omegaP_i", C.c_double * MAXP), ("GammaP_i", C.c_double * MAXP), ("AP_i", C.c_double * MAXP)]


class OrcConstants(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("pi0", "c0", "eps0", "mu0", "sec_to_au", "C_to_au", "kg_to_au",
                                          "m_to_au", "nm_to_au", "au_to_nm", "ev_to_au", "au_to_ev",
                                          "Debye_to_au", "fs_to_au", "au_to_fs", "alphaCPML", "kappaCPML")]
    _fields_ += [("aBH", C.c_double * 4), ("sig_to_au", C.c_double)]


class OrcSourceDesc(C.Structure):
    _fields_ = [("dir", C.c_char), ("j_amp", C.c_double), ("w0", C.c_double), ("t0", C.c_double),
                ("tau", C.c_double), ("t_init", C.c_double), ("t_final", C.c_double),
                ("phase", C.c_double), ("r0", C.c_double * 3), ("rad", C.c_double), ("chirp", C.c_double)]


class OrcPlaneDesc(C.Structure):
    _fields_ = [("comp", C.c_int), ("plane_axis", C.c_int), ("plane_idx", C.c_int),
                ("j_amp", C.c_double), ("w0", C.c_double), ("t0", C.c_double), ("tau", C.c_double),
                ("t_init", C.c_double), ("t_final", C.c_double), ("phase", C.c_double), ("chirp", C.c_double)]


_PD = C.POINTER(C.c_double)
_P32 = C.POINTER(C.c_int32)
_PI = C.POINTER(C.c_int)
_VP = C.c_void_p


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError(f"{LIB} missing: run oracle/build_oracle.py")
        L = C.CDLL(LIB)
        sig = {
            "orc_get_constants": (None, [C.POINTER(OrcConstants)]),
            "orc_medium_dielectric": (None, [C.c_double, C.POINTER(OrcMedium)]),
            "orc_medium_drude": (None, [C.c_double, C.c_double, C.c_double, C.c_double, C.POINTER(OrcMedium)]),
            "orc_medium_dl_library": (C.c_int, [C.c_char_p, C.c_double, C.c_double, C.POINTER(OrcMedium)]),
            "orc_medium_dl_custom": (None, [C.c_double, C.c_double, C.c_double, C.c_int, _PD, _PD, _PD,
                                            C.c_double, C.POINTER(OrcMedium)]),
            "orc_cpml_tables": (None, [C.c_int, C.c_double, C.c_double, _PD, _PD, _PD, _PD, _PD, _PD]),
            "orc_media_map_3d": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, _PI, _PD, _P32]),
            "orc_media_map_2d": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_int, _PI, _PD, _P32]),
            "orc_media_map_1d": (C.c_int, [C.c_int, C.c_double, C.c_int, _PI, _PD, _P32]),
            "orc_grid_create": (_VP, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _PI, C.c_int, C.c_double,
                                      C.c_double]),
            "orc_grid_destroy": (None, [_VP]),
            "orc_grid_set_media": (C.c_int, [_VP, C.c_int, C.POINTER(OrcMedium), _P32, _PD, _PD, _PD]),
            "orc_grid_set_time": (None, [_VP, C.c_double, C.c_double]),
            "orc_propagate_H": (None, [_VP]),
            "orc_propagate_E": (None, [_VP]),
            "orc_field_size": (C.c_long, [_VP, C.c_int]),
            "orc_field_get": (C.c_long, [_VP, C.c_int, _PD]),
            "orc_field_set": (C.c_long, [_VP, C.c_int, _PD]),
            "orc_field_bounds": (C.c_int, [_VP, C.c_int, _PI, _PI]),
            "orc_source_create": (_VP, [_VP, C.POINTER(OrcSourceDesc)]),
            "orc_source_destroy": (None, [_VP]),
            "orc_source_update": (None, [_VP, C.c_double]),
            "orc_source_interactions": (None, [_VP, C.POINTER(_VP), C.c_int]),
            "orc_source_kernel": (C.c_int, [_VP, _PD, _PI]),
            "orc_plane_source_apply": (None, [_VP, C.POINTER(OrcPlaneDesc), C.c_double]),
            "orc_qgroup_create": (_VP, [_VP, C.c_int, C.c_int, C.c_int, _P32, _PD, C.c_double, C.c_double]),
            "orc_qgroup_destroy": (None, [_VP]),
            "orc_send_E_to_J": (None, [_VP, _VP]),
            "orc_td_propagate_q_group": (None, [_VP, C.c_int]),
            "orc_send_J_to_E": (None, [_VP, _VP]),
            "orc_qgroup_read": (None, [_VP, _PD, _PD, _PD, _PD]),
            "orc_qgroup_state_size": (C.c_int, [_VP]),
            "orc_emitter_step": (None, [C.c_int, _PD, _PD, C.c_double, C.c_double]),
            "orc_sample": (None, [_VP, C.c_int, C.c_int, C.c_int, _P32, _PD]),
            "orc_num_threads": (C.c_int, []),
            "fd_create": (_VP, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _PI, C.c_double, C.c_double,
                                _PD]),
            "fd_destroy": (None, [_VP]),
            "fd_vec_len": (C.c_longlong, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
            "fd_apply": (None, [_VP, _PD, _PD, C.c_int]),
            "fd_bicgstab_l": (C.c_int, [_VP, _PD, _PD, C.c_int, C.c_double, C.c_int, C.c_int, _PI, _PD]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_PD)


def constants():
    c = OrcConstants()
    lib().orc_get_constants(C.byref(c))
    return c


def cpml_tables(npml, dr, dt):
    be, ce, ke = np.zeros(npml), np.zeros(npml), np.zeros(npml)
    bh, ch, kh = np.zeros(npml - 1), np.zeros(npml - 1), np.zeros(npml - 1)
    lib().orc_cpml_tables(npml, dr, dt, _d(be), _d(ce), _d(bh), _d(ch), _d(ke), _d(kh))
    return be, ce, bh, ch, ke, kh


def medium_dielectric(eps_r):
    m = OrcMedium()
    lib().orc_medium_dielectric(eps_r, C.byref(m))
    return m


def medium_drude(omegaD, GammaD, eps_r, dt):
    m = OrcMedium()
    lib().orc_medium_drude(omegaD, GammaD, eps_r, dt, C.byref(m))
    return m


def medium_dl_library(name, eps_r, dt):
    m = OrcMedium()
    if lib().orc_medium_dl_library(name.encode(), eps_r, dt, C.byref(m)) != 0:
        raise ValueError(name)
    return m


def medium_dl_custom(eps_inf, wp, gamma, poles, strengths, widths, dt):
    m = OrcMedium()
    p, s, w = (np.ascontiguousarray(x, dtype=np.float64) for x in (poles, strengths, widths))
    lib().orc_medium_dl_custom(eps_inf, wp, gamma, len(p), _d(p), _d(s), _d(w), dt, C.byref(m))
    return m


def media_map(dims, n, dr, voxels_per_medium):
    counts = np.array([len(v) for v in voxels_per_medium], dtype=np.int32)
    vox = (np.ascontiguousarray(np.concatenate([np.asarray(v, np.float64).reshape(-1, dims)
                                                for v in voxels_per_medium]).reshape(-1))
           if counts.sum() else np.zeros(1))
    if dims == 3:
        out = np.zeros(n[0] * n[1] * n[2] * 3, np.int32)
        lib().orc_media_map_3d(n[0], n[1], n[2], dr, len(counts), counts.ctypes.data_as(_PI), _d(vox),
                               out.ctypes.data_as(_P32))
        return out.reshape((n[0], n[1], n[2], 3), order="F")
    if dims == 2:
        out = np.zeros(n[0] * n[1] * 3, np.int32)
        lib().orc_media_map_2d(n[0], n[1], dr, len(counts), counts.ctypes.data_as(_PI), _d(vox),
                               out.ctypes.data_as(_P32))
        return out.reshape((n[0], n[1], 3), order="F")
    out = np.zeros(n[0], np.int32)
    lib().orc_media_map_1d(n[0], dr, len(counts), counts.ctypes.data_as(_PI), _d(vox), out.ctypes.data_as(_P32))
    return out


def emitter_step(model, params, rho, E_u, dt):
    p = np.ascontiguousarray(params, dtype=np.float64)
    r = np.ascontiguousarray(rho, dtype=np.float64).copy()
    lib().orc_emitter_step(int(model), _d(p), _d(r), float(E_u), float(dt))
    return r


class Grid:
    """The oracle's TMxll: same call sequence as the GPU TMxll wrapper."""

    def __init__(self, dimensions, grid_Ndims, npml, boundaries, dt, dr, mode=1):
        g = list(grid_Ndims) + [1] * (3 - len(grid_Ndims))
        b = (C.c_int * 3)(*(list(boundaries) + [1] * (3 - len(boundaries))))
        self.dimensions = dimensions
        self.dt, self.dr = dt, dr
        self._g = lib().orc_grid_create(dimensions, g[0], g[1], g[2], npml, b, mode, dt, dr)
        self._src = []
        self._groups = []
        self._planes = []

    def __del__(self):
        try:
            for s in self._src:
                lib().orc_source_destroy(s)
            for q in self._groups:
                lib().orc_qgroup_destroy(q[0])
            lib().orc_grid_destroy(self._g)
        except Exception:
            pass

    def set_media(self, media, media_map_arr, eps=None):
        arr = (OrcMedium * max(1, len(media)))(*media) if media else (OrcMedium * 1)()
        mm = np.ascontiguousarray(np.asarray(media_map_arr).reshape(-1, order="F"), dtype=np.int32)
        e = [None, None, None]
        if eps is not None:
            e = [np.ascontiguousarray(np.asarray(x).reshape(-1, order="F"), np.float64) if x is not None else None
                 for x in eps]
        lib().orc_grid_set_media(self._g, len(media), arr, mm.ctypes.data_as(_P32),
                                 *[(_d(x) if x is not None else None) for x in e])

    def set_time(self, time, t_skip):
        lib().orc_grid_set_time(self._g, time, t_skip)

    def td_propagate_H_field(self):
        lib().orc_propagate_H(self._g)

    def td_propagate_E_field(self, time, t_skip):
        lib().orc_grid_set_time(self._g, time, t_skip)
        lib().orc_propagate_E(self._g)

    def add_source(self, direction, j_amp, w0, t0, tau, r0, radius, t_init, t_final, phase=0.0, chirp=0.0):
        d = OrcSourceDesc()
        d.dir = direction.encode()
        d.j_amp, d.w0, d.t0, d.tau, d.t_init, d.t_final, d.phase = j_amp, w0, t0, tau, t_init, t_final, phase
        d.r0 = (C.c_double * 3)(*[float(v) for v in list(r0) + [0.0] * (3 - len(r0))])
        d.rad, d.chirp = radius, chirp
        s = lib().orc_source_create(self._g, C.byref(d))
        self._src.append(s)
        return s

    def add_plane_source(self, comp, plane_axis, plane_index, j_amp, w0, t0, tau, t_init, t_final, phase=0.0,
                         chirp=0.0):
        d = OrcPlaneDesc()
        d.comp, d.plane_axis, d.plane_idx = comp, plane_axis, plane_index
        d.j_amp, d.w0, d.t0, d.tau, d.t_init, d.t_final, d.phase, d.chirp = (
            j_amp, w0, t0, tau, t_init, t_final, phase, chirp)
        self._planes.append(d)

    def source_interactions(self, time):
        for s in self._src:
            lib().orc_source_update(s, time)
        if self._src:
            arr = (C.c_void_p * len(self._src))(*self._src)
            lib().orc_source_interactions(self._g, arr, len(self._src))
        for d in self._planes:
            lib().orc_plane_source_apply(self._g, C.byref(d), time)

    def add_q_group(self, group_type, model, cells, params, density, dt):
        cells = np.ascontiguousarray(np.asarray(cells, dtype=np.int32).reshape(-1))
        params = np.ascontiguousarray(np.asarray(params, dtype=np.float64).reshape(-1))
        n = len(cells) // self.dimensions
        q = lib().orc_qgroup_create(self._g, group_type, model, n, cells.ctypes.data_as(_P32), _d(params),
                                    density, dt)
        self._groups.append((q, n))
        return len(self._groups) - 1

    def q_group_step(self, gid, tq_step=1):
        q = self._groups[gid][0]
        lib().orc_send_E_to_J(self._g, q)
        lib().orc_td_propagate_q_group(q, tq_step)
        lib().orc_send_J_to_E(self._g, q)

    def q_group_read(self, gid):
        q, n = self._groups[gid]
        nst = lib().orc_qgroup_state_size(q)
        dip, dpdt, ef, rho = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, nst))
        lib().orc_qgroup_read(q, _d(dip), _d(dpdt), _d(ef), _d(rho))
        return {"dipole": dip, "dPt_dt": dpdt, "E": ef, "rho": rho}

    def field_bounds(self, field):
        lo, hi = (C.c_int * 3)(), (C.c_int * 3)()
        if lib().orc_field_bounds(self._g, field, lo, hi) != 0:
            raise KeyError(field)
        return list(lo), list(hi)

    def read_field(self, field):
        lo, hi = self.field_bounds(field)
        shape = tuple(hi[a] - lo[a] + 1 for a in range(3))
        out = np.zeros(int(np.prod(shape)))
        lib().orc_field_get(self._g, field, _d(out))
        return out.reshape(shape, order="F")

    def write_field(self, field, values):
        flat = np.ascontiguousarray(np.asarray(values).reshape(-1, order="F"), np.float64)
        lib().orc_field_set(self._g, field, _d(flat))

    def sample(self, detector_type, field, indx_list):
        idx = np.asarray(indx_list, dtype=np.int32).reshape(-1, self.dimensions)
        flat = np.ascontiguousarray(idx.reshape(-1, order="F"))
        out = np.zeros(idx.shape[0])
        lib().orc_sample(self._g, detector_type, field, idx.shape[0], flat.ctypes.data_as(_P32), _d(out))
        return out


def fd_shape(n, n_der):
    """Array shape of a frequency-domain vector on grid n (1, 2 or 3 sizes): 3D [6][nz+2g][ny+2g]
    [nx+2g], 2D [6][ny+2g][nx+2g], 1D [4][nx+2g] (components pl_x, pl_y, (pl_z,) mi_x, mi_y,
    (mi_z); g = n_der ghost cells on each side of every axis)."""
    g = n_der
    pad = tuple(v + 2 * g for v in reversed(n))
    return ((4,) if len(n) == 1 else (6,)) + pad


class FDOperator:
    """The frequency-domain operator and its BiCGStab(L) solver (fd_oracle.c) on a 1D, 2D or 3D
    grid n; vectors as fd_shape describes, eps_r of shape n."""

    def __init__(self, n, n_pml, n_der, boundaries, dr, w0, eps):
        self.n, self.g = tuple(int(v) for v in n), n_der
        dims = len(self.n)
        nn = list(self.n) + [1] * (3 - dims)
        eps = np.ascontiguousarray(np.asarray(eps, np.complex128).reshape(self.n).transpose())   # x fastest
        b = np.asarray(list(boundaries) + [1] * (3 - len(boundaries)), np.int32)
        self._h = lib().fd_create(dims, nn[0], nn[1], nn[2], n_pml, n_der, b.ctypes.data_as(_PI), float(dr),
                                  float(w0), eps.view(np.float64).ctypes.data_as(_PD))

    def shape(self):
        return fd_shape(self.n, self.g)

    def zeros(self):
        return np.zeros(self.shape(), np.complex128)

    def apply(self, f, transpose=False):
        f = np.ascontiguousarray(f, np.complex128).copy()
        out = self.zeros()
        lib().fd_apply(self._h, f.view(np.float64).ctypes.data_as(_PD), out.view(np.float64).ctypes.data_as(_PD),
                       1 if transpose else 0)
        return out

    def solve(self, j, f0, tol, n_max, L, transpose=False):
        j = np.ascontiguousarray(j, np.complex128)
        f = np.ascontiguousarray(f0, np.complex128).copy()
        conv = C.c_int()
        err = C.c_double()
        it = lib().fd_bicgstab_l(self._h, j.view(np.float64).ctypes.data_as(_PD),
                                 f.view(np.float64).ctypes.data_as(_PD), 1 if transpose else 0, float(tol), int(n_max),
                                 int(L), C.byref(conv), C.byref(err))
        return f, bool(conv.value), err.value, it

    def __del__(self):
        try:
            lib().fd_destroy(self._h)
        except Exception:
            pass
