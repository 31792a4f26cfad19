"""Detector outputs built on the device state: FP64 running Fourier transforms of the samples,
the field energy, and the reference-layout text writers (detector files, energy_and_dipole.dat)."""
import os

import numpy as np
import pytest

import omx
from omx import decks
from gpu_harness import tmz_variant_deck

pytestmark = pytest.mark.gpu


def _tmz(precision="fp64", with_groups=True):
    deck = tmz_variant_deck(96, 64, 2, 3, src="radial")
    g = omx.TMxll(2, deck["grid_Ndims"], deck["npml"], deck["boundaries"], deck["dt"], deck["dr"], mode=omx.TMZ,
                  precision=precision)
    groups = decks.apply_deck(g, deck, omx, decks.media_map(deck, omx.media_map_from_voxels))
    for det in deck["detectors"]:
        g.add_detector(det["type"], det["field"], det["idx"])
    return deck, g, groups


@pytest.mark.parametrize("graph", [True, False])
def test_dft_accumulators_match_numpy(graph):
    deck, g, _ = _tmz()
    ev = omx.UNITS["ev_to_au"]
    omega = np.array([1.5, 2.8, 3.3]) * ev
    g.dft_setup(omega, deck["dt"])
    g.run(1, 150, deck["n_skip"], 1, use_graph=graph)
    times, trace = g.drain_detectors()
    F = g.dft_read()
    ref = np.zeros_like(F)
    for k, w in enumerate(omega):
        ref[k] = deck["dt"] * ((trace * np.cos(w * times)[:, None]).sum(0) - 1j * (trace * np.sin(w * times)[:, None]).sum(0))
    scale = np.max(np.abs(ref))
    assert scale > 0
    assert np.max(np.abs(F - ref)) <= 1e-12 * scale
    g.kill()


def test_field_energy_matches_numpy():
    deck, g, _ = _tmz(with_groups=False)
    g.run(1, 120, deck["n_skip"], 0, use_graph=True)
    e = g.field_energy()
    n = deck["grid_Ndims"]
    tot = 0.0
    for f, const in ((3, omx.UNITS["eps0"]), (4, omx.UNITS["mu0"]), (5, omx.UNITS["mu0"])):
        a = g.read_field(f)
        lo, _ = g.field_bounds(f)
        a = a[1 - lo[0]:n[0] + 1 - lo[0], 1 - lo[1]:n[1] + 1 - lo[1]]
        tot += const * np.sum(a * a)
    ref = 0.5 * deck["dr"] ** 2 * tot
    assert ref > 0 and abs(e - ref) <= 1e-12 * ref
    g.kill()


def test_text_writers(tmp_path):
    deck, g, groups = _tmz()
    deck2, g2, _ = _tmz()
    plane = np.stack(np.meshgrid(np.arange(20, 30), np.arange(30, 36), indexing="ij"), -1).reshape(-1, 2)
    for gg in (g, g2):
        gg.add_detector(omx.PLANE_XY, 3, plane.astype(np.int32))
        gg.run(1, 40, deck["n_skip"], 4, use_graph=True)
    times, trace = g2.drain_detectors()
    nrec = g.write_detectors_text(tmp_path)
    assert nrec == len(times) == 10
    npts_det = [1] * len(deck["detectors"])
    # point detectors: "time value" per record, values as drained (17 significant digits)
    for d in range(len(deck["detectors"])):
        rows = np.loadtxt(os.path.join(tmp_path, f"output_detector_{d + 1:07d}", "point.dat"))
        assert np.array_equal(rows[:, 0], times) and np.array_equal(rows[:, 1], trace[:, d])
    # the plane: one file per record, a header and one line per cell (x, y in nm, value)
    dd = len(deck["detectors"]) + 1
    first = sum(npts_det)
    for r in range(nrec):
        f = os.path.join(tmp_path, f"output_detector_{dd:07d}", f"Ez_plane_{r:09d}.dat")
        with open(f) as fh:
            assert fh.readline().startswith("# Time =")
        rows = np.loadtxt(f)
        assert rows.shape == (plane.shape[0], 3)
        assert np.array_equal(rows[:, 2], trace[r, first:first + plane.shape[0]])
        x_nm = (plane[:, 0] * deck["dr"] - (deck["grid_Ndims"][0] // 2) * deck["dr"]) * omx.UNITS["au_to_nm"]
        assert np.allclose(rows[:, 0], x_nm, rtol=1e-6, atol=0)     # au_to_nm is a single-precision literal
    # q-group energy_and_dipole.dat: one line per emitter, energy = w0 * p_e in eV
    groups[0].write_text(tmp_path, times[-1])
    rows = np.loadtxt(os.path.join(tmp_path, "output_q_group_0001", "energy_and_dipole.dat"))
    st = groups[0].read()
    par = np.asarray(deck["groups"][0]["params"])
    assert rows.shape == (par.shape[0], 5)
    assert np.allclose(rows[:, 1], par[:, 0] * st["rho"][:, 0] * float(np.float32(27.2114)), rtol=1e-15, atol=0)
    assert np.array_equal(rows[:, 2:], st["dipole"])
    g.kill()
    g2.kill()
