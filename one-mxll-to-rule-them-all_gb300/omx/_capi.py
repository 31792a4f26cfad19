"""ctypes declarations of include/omx_gpu.h.

The library is loaded from the package directory; there is no fallback: a missing or
unloadable libomx_gpu.so raises OMXError.
"""
import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "libomx_gpu.so")

OMX_OK = 0
CLOSE, PERIODIC, CPML = 1, 2, 3
TMZ, TEZ = 1, 2
NONE_MEDIUM, DIELECTRIC, DRUDE, DL = 0, 1, 2, 3
EX, EY, EZ, HX, HY, HZ = 1, 2, 3, 4, 5, 6
FIELDS = {"Ex": EX, "Ey": EY, "Ez": EZ, "Hx": HX, "Hy": HY, "Hz": HZ}
POINT, LINE_X, LINE_Y, LINE_Z, PLANE_XY, PLANE_YZ, PLANE_ZX, VOLUME = range(1, 9)
Q_MATERIAL, Q_SINGLE = 1, 2
PREC_FP64, PREC_FP32 = 0, 1
TWO_LEVEL, THREE_LEVEL = 1, 2
MAX_POLES = 8
KC_H, KC_E, KC_EMIT, KC_SRC, KC_DET = range(5)
STEP_DEFAULT, STEP_TWO_PASS, STEP_SINGLE_PASS = 0, 1, 2


class OMXError(RuntimeError):
    pass


class GridDesc(C.Structure):
    _fields_ = [("dimensions", C.c_int), ("grid_Ndims", C.c_int * 3), ("npml", C.c_int),
                ("boundaries", C.c_int * 3), ("mode", C.c_int), ("precision", C.c_int),
                ("dt", C.c_double), ("dr", C.c_double)]


class Medium(C.Structure):
    _fields_ = [("medium_type", C.c_int), ("n_poles", C.c_int), ("eps_r", C.c_double),
                ("A1", C.c_double), ("A2", C.c_double), ("C1", C.c_double), ("C2", C.c_double),
                ("C3", C.c_double), ("C4", C.c_double),
                ("alpha_k", C.c_double * MAX_POLES), ("beta_k", C.c_double * MAX_POLES),
                ("gamma_k", C.c_double * MAX_POLES), ("B1_k", C.c_double * MAX_POLES),
                ("B2_k", C.c_double * MAX_POLES)]


class SourceDesc(C.Structure):
    _fields_ = [("dir", C.c_char), ("j_amp", C.c_double), ("w0", C.c_double), ("t0", C.c_double),
                ("tau", C.c_double), ("t_init", C.c_double), ("t_final", C.c_double),
                ("phase", C.c_double), ("r0", C.c_double * 3), ("radius", C.c_double),
                ("chirp", C.c_double)]


class PlaneSourceDesc(C.Structure):
    _fields_ = [("comp", C.c_int), ("plane_axis", C.c_int), ("plane_index", C.c_int),
                ("j_amp", C.c_double), ("w0", C.c_double), ("t0", C.c_double), ("tau", C.c_double),
                ("t_init", C.c_double), ("t_final", C.c_double), ("phase", C.c_double),
                ("chirp", C.c_double)]


class QGroupDesc(C.Structure):
    _fields_ = [("group_type", C.c_int), ("model", C.c_int), ("n_systems", C.c_int),
                ("density", C.c_double), ("dt", C.c_double)]


_VP = C.c_void_p
_I = C.c_int
_D = C.c_double
_PD = C.POINTER(C.c_double)
_PI = C.POINTER(C.c_int)
_P32 = C.POINTER(C.c_int32)
_PF = C.POINTER(C.c_float)

SIGNATURES = {
    "omx_select_device": (_I, [_I]),
    "omx_device_count": (_I, [_PI]),
    "omx_create": (_I, [C.POINTER(GridDesc), C.POINTER(_VP)]),
    "omx_destroy": (_I, [_VP]),
    "omx_last_error": (C.c_char_p, [_VP]),
    "omx_synchronize": (_I, [_VP]),
    "omx_get_cpml_tables": (_I, [_VP, _PD, _PD, _PD, _PD]),
    "omx_get_den": (_I, [_VP, _I, _PD, _PD]),
    "omx_compute_cpml_tables": (_I, [_I, _D, _D, _PD, _PD, _PD, _PD, _PD, _PD]),
    "omx_set_cpml_tables": (_I, [_VP, _PD, _PD, _PD, _PD, _PD, _PD, _PD, _PD, _PD, _PD]),
    "omx_set_media": (_I, [_VP, _I, C.POINTER(Medium), _P32, _PD, _PD, _PD]),
    "omx_medium_dielectric": (_I, [_D, C.POINTER(Medium)]),
    "omx_medium_drude": (_I, [_D, _D, _D, _D, C.POINTER(Medium)]),
    "omx_medium_dl_library": (_I, [C.c_char_p, _D, _D, C.POINTER(Medium)]),
    "omx_medium_dl_custom": (_I, [_D, _D, _D, _I, _PD, _PD, _PD, _D, C.POINTER(Medium)]),
    "omx_media_map_from_voxels": (_I, [_I, _PI, _D, _I, _PI, _PD, _P32]),
    "omx_step_H": (_I, [_VP]),
    "omx_step_E": (_I, [_VP, _D, _D]),
    "omx_source_add": (_I, [_VP, C.POINTER(SourceDesc), _PI]),
    "omx_plane_source_add": (_I, [_VP, C.POINTER(PlaneSourceDesc), _PI]),
    "omx_source_interactions": (_I, [_VP, _D]),
    "omx_qgroup_create": (_I, [_VP, C.POINTER(QGroupDesc), _P32, _PD, _PI]),
    "omx_qgroup_step": (_I, [_VP, _I, _I]),
    "omx_qgroup_read": (_I, [_VP, _I, _PD, _PD, _PD, _PD]),
    "omx_qgroup_state_size": (_I, [_I]),
    "omx_emitter_step_noalloc": (_I, [_I, _I, _VP, _VP, _VP, _VP, _I, _VP, _VP, _VP, _VP, _VP, _I, _I, _D, _VP]),
    "omx_detector_add": (_I, [_VP, _I, _I, _I, _P32, _PI]),
    "omx_detectors_total_points": (_I, [_VP]),
    "omx_detectors_set_capacity": (_I, [_VP, _I]),
    "omx_detectors_record": (_I, [_VP, _D]),
    "omx_detectors_drain": (_I, [_VP, _PD, _PD, _I, _PI]),
    "omx_detectors_drain_async": (_I, [_VP, C.POINTER(C.c_longlong)]),
    "omx_set_step_form": (_I, [_VP, _I]),
    "omx_detectors_collect": (_I, [_VP, C.c_longlong, _PD, _PD, _I, _PI]),
    "omx_run": (_I, [_VP, _I, _I, _I, _I, _I]),
    "omx_run_prepare": (_I, [_VP, _I, _I, _I, _I]),
    "omx_set_launch_shape": (_I, [_VP, _I]),
    "omx_detectors_write_text": (_I, [_VP, C.c_char_p, _PI]),
    "omx_detectors_dft_setup": (_I, [_VP, _I, _PD, _D]),
    "omx_detectors_dft_read": (_I, [_VP, _PD, _PD]),
    "omx_field_energy": (_I, [_VP, _PD]),
    "omx_qgroup_write_text": (_I, [_VP, _I, C.c_char_p, _D, _I]),
    "omx_autotune": (_I, [_VP, _I, _PI]),
    "omx_batch_create": (_I, [C.POINTER(_VP), _I, C.POINTER(_VP)]),
    "omx_batch_autotune": (_I, [_VP, _I, _PI]),
    "omx_batch_set_launch_shape": (_I, [_VP, _I]),
    "omx_batch_run": (_I, [_VP, _I, _I, _I, _I, _I]),
    "omx_batch_run_prepare": (_I, [_VP, _I, _I, _I, _I]),
    "omx_batch_launch_count": (C.c_longlong, [_VP]),
    "omx_batch_synchronize": (_I, [_VP]),
    "omx_tc_gemm_bf16": (_I, [C.POINTER(C.c_uint16), C.POINTER(C.c_uint16), _PF, _PF, _I, _I, _I, C.c_float, _I]),
    "omx_closure_create": (_I, [C.POINTER(_VP)]),
    "omx_closure_destroy": (_I, [_VP]),
    "omx_closure_n_params": (C.c_longlong, []),
    "omx_closure_set_params": (_I, [_VP, _PF, _D, _D]),
    "omx_closure_get_params": (_I, [_VP, _PF, _PD, _PD]),
    "omx_closure_forward": (_I, [_VP, _PF, _I, _I, _PF]),
    "omx_closure_gradient": (_I, [_VP, _PF, _PF, _I, _I, _I, _PF, _PD]),
    "omx_closure_train_step": (_I, [_VP, _PF, _PF, _I, _I, _I, C.c_float, _PD]),
    "omx_closure_trajectories": (_I, [_I, _I, _I, _I, _D, _PD, _PD, _D, _D, _PF, _PF]),
    "omx_qgroup_attach_closure": (_I, [_VP, _I, _VP, _D, _D, _I]),
    "omx_qgroup_closure_status": (_I, [_VP, _I, _PD, _PI, _PI, _PI]),
    "omx_fd_create": (_I, [_I, _PI, _I, _I, _PI, _D, _D, _PD, C.POINTER(_VP)]),
    "omx_fd_destroy": (_I, [_VP]),
    "omx_fd_vector_length": (C.c_longlong, [_VP]),
    "omx_fd_apply": (_I, [_VP, _PD, _PD, _I]),
    "omx_fd_solve": (_I, [_VP, _PD, _PD, _I, _D, _I, _I, _PI, _PD, _PI]),
    "omx_fd_time_apply": (_I, [_VP, _I, _PD]),
    "omx_fd_set_eps": (_I, [_VP, _PD]),
    "omx_batch_destroy": (_I, [_VP]),
    "omx_field_bounds": (_I, [_VP, _I, _PI, _PI]),
    "omx_read_field": (_I, [_VP, _I, _PD]),
    "omx_write_field": (_I, [_VP, _I, _PD]),
    "omx_profile_enable": (_I, [_VP, _I]),
    "omx_profile_query": (_I, [_VP, _I, _PD, C.POINTER(C.c_longlong)]),
    "omx_algorithmic_bytes": (_I, [_VP, _I, _PD]),
    "omx_launch_count": (C.c_longlong, [_VP]),
    "omx_timer_start": (_I, [_VP]),
    "omx_timer_stop": (_I, [_VP, C.POINTER(C.c_float)]),
    "omx_flush_l2": (_I, [_VP]),
}

_lib = None


def lib():
    """Load libomx_gpu.so (raises OMXError when it is missing: there is no CPU path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OMXError(f"{LIB_PATH} is missing: build it with one-mxll-to-rule-them-all_gb300/build.py")
    try:
        L = C.CDLL(LIB_PATH)
    except OSError as e:
        raise OMXError(f"cannot load {LIB_PATH}: {e}") from e
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc, ctx=None):
    if rc != OMX_OK:
        msg = lib().omx_last_error(ctx)
        raise OMXError(f"omx status {rc}: {msg.decode() if msg else ''}")


def dptr(a):
    return a.ctypes.data_as(_PD) if a is not None else None


def iptr(a):
    return a.ctypes.data_as(_P32) if a is not None else None


def as_f64(a):
    return np.ascontiguousarray(a, dtype=np.float64) if a is not None else None


def fortran_flat_i32(a):
    """Flatten an array given in Fortran index order (first index fastest) to int32."""
    a = np.asarray(a)
    return np.ascontiguousarray(a.reshape(-1, order="F"), dtype=np.int32)


def fortran_flat_f64(a):
    a = np.asarray(a)
    return np.ascontiguousarray(a.reshape(-1, order="F"), dtype=np.float64)
