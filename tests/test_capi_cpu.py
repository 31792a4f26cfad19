"""C-ABI checks that need no GPU: the library loads, exports every entry point declared in
include/omx_gpu.h, reproduces the oracle's set-up arithmetic bit for bit, and refuses to run
without a CUDA device (there is no CPU path)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared_entry_points():
    src = open(os.path.join(ROOT, "include", "omx_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(omx_[A-Za-z0-9_]+)\s*\(", src)))


def test_header_symbols_exported(omx):
    names = _declared_entry_points()
    assert len(names) >= 39
    L = omx.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_python_binding_covers_header(omx):
    from omx import _capi

    names = _declared_entry_points()
    assert set(names) <= set(_capi.SIGNATURES), sorted(set(names) - set(_capi.SIGNATURES))


def test_no_gpu_fails_loudly(omx):
    import subprocess
    import sys

    code = ("import sys; sys.path.insert(0, %r); import omx\n"
            "try:\n    omx.TMxll(3, (8, 8, 8), 2, (1, 1, 1), 0.1, 1.0)\nexcept omx.OMXError as e:\n"
            "    print('ERR', e)\nelse:\n    print('OK')\n") % os.path.join(ROOT, "one-mxll-to-rule-them-all_gb300")
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env).stdout
    assert out.startswith("ERR") and "no CUDA device" in out


@pytest.mark.parametrize("npml,dr_nm", [(10, 2.0), (8, 20.0), (19, 1.0), (2, 1.0)])
def test_cpml_tables_match_oracle(omx, orc, npml, dr_nm):
    dr = dr_nm * omx.UNITS["nm_to_au"]
    dt = dr / 274.0
    a = omx.compute_cpml_tables(npml, dr, dt)
    b = orc.cpml_tables(npml, dr, dt)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def _medium_fields(m):
    vals = [m.medium_type, m.eps_r, m.A1, m.A2, m.C1, m.C2, m.C3, m.C4]
    n = m.n_poles if m.medium_type == 3 else 0
    for f in ("alpha_k", "beta_k", "gamma_k", "B1_k", "B2_k"):
        vals += list(getattr(m, f))[:n]
    return vals


def test_medium_coefficients_match_oracle(omx, orc):
    ev = omx.UNITS["ev_to_au"]
    dt = 2.0 * omx.UNITS["nm_to_au"] / 274.0
    pairs = [
        (omx.medium_drude(9.17 * ev, 0.021 * ev, 1.0, dt), orc.medium_drude(9.17 * ev, 0.021 * ev, 1.0, dt)),
        (omx.medium_dielectric(12.1), orc.medium_dielectric(12.1)),
        (omx.medium_dl_custom(5.9, 9.0, 0.07, [2.7, 3.9], [1.0, 0.6], [0.3, 0.5], dt),
         orc.medium_dl_custom(5.9, 9.0, 0.07, [2.7, 3.9], [1.0, 0.6], [0.3, 0.5], dt)),
    ]
    for name in ("Ag", "Al", "Au"):
        pairs.append((omx.medium_dl_library(name, 1.0, dt), orc.medium_dl_library(name, 1.0, dt)))
    for a, b in pairs:
        assert _medium_fields(a) == _medium_fields(b)
    with pytest.raises(omx.OMXError):
        omx.medium_dl_library("Cu", 1.0, dt)


def test_media_map_rule_matches_oracle(omx, orc):
    rng = np.random.default_rng(11)
    # 3D: two overlapping random blobs, including cells on the last planes
    n = (12, 10, 9)
    dr = 2.0 * omx.UNITS["nm_to_au"]
    vox = []
    for m in range(2):
        cells = rng.integers(1, np.array(n) + 1, size=(150, 3))
        vox.append(np.stack([((c - nn // 2) + np.where(c - nn // 2 >= 0, 0.5, -0.5)) * 2.0
                             for c, nn in zip(cells.T, n)], axis=1))
    a = omx.media_map_from_voxels(3, n, dr, vox)
    b = orc.media_map(3, n, dr, vox)
    assert a.shape == b.shape and np.array_equal(a, b) and a.max() == 2
    # 2D and 1D
    n2 = (14, 11)
    vox2 = [np.stack([((c - nn // 2) + np.where(c - nn // 2 >= 0, 0.5, -0.5)) * 2.0
                      for c, nn in zip(rng.integers(1, np.array(n2) + 1, size=(60, 2)).T, n2)], axis=1)]
    assert np.array_equal(omx.media_map_from_voxels(2, n2, dr, vox2), orc.media_map(2, n2, dr, vox2))
    vox1 = [rng.uniform(-20, 20, size=(9, 1))]
    assert np.array_equal(omx.media_map_from_voxels(1, (30,), dr, vox1), orc.media_map(1, (30,), dr, vox1))


def test_deck_media_maps_match(omx, orc):
    from omx import decks

    for d in (decks.deck_cfg1(n=40, radius_nm=12.0), decks.deck_cfg2(nx=300, ny=120, n_emitters=50),
              decks.deck_cfg3(n=96, n_emitters=200), decks.deck_cfg5_instance(32, seed=3)):
        a = decks.media_map(d, omx.media_map_from_voxels)
        b = decks.media_map(d, lambda dims, n, dr, v: orc.media_map(dims, n, dr, v))
        assert np.array_equal(a, b)
        assert a.max() >= 1
        for det in d["detectors"]:
            assert det["idx"].shape == (1, d["dimensions"])
