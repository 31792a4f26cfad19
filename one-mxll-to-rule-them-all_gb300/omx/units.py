"""Unit conversions with the reference's literal precision (src/FDTD/constants_mod.f90:31-49).

Default-real Fortran literals are single precision, so several "double" constants are values
rounded to float32 first; the deck-building code needs the same numbers as the reference.
"""
import numpy as np

_pi0 = 3.141592653589793
_eps0 = 1.0 / (4.0 * _pi0)

UNITS = {
    "pi0": _pi0,
    "c0": 137.0,
    "eps0": _eps0,
    "mu0": 1.0 / (_eps0 * (137.0 * 137.0)),
    "nm_to_au": float(np.float32(18.897261259077823)),
    "ev_to_au": float(np.float32(1.0) / np.float32(27.2114)),
    "au_to_ev": float(np.float32(27.2114)),
    "Debye_to_au": float(np.float32(3.0) / np.float32(7.63)),
    "fs_to_au": 1.0 / 2.4188843265864e-2,
    "au_to_fs": 2.4188843265864e-2,
}
UNITS["au_to_nm"] = 1.0 / UNITS["nm_to_au"]
# atomic unit of electric field in V/m (for drive amplitudes quoted in V/m)
UNITS["Vm_to_au"] = 1.0 / 5.14220674763e11


def yee_dt(dr_au):
    """dt = MIN(dr/(2*c0), mxll_dt) with the default mxll_dt (input_mod.f90:122)."""
    return min(dr_au / (2.0 * 137.0), 10.0e10)
