"""GPU parity: the CUDA library (through its C-ABI) against the CPU FP64 oracle on the same
seeded decks.

FP64 plain path: bit-identical fields, detector samples and emitter dipoles (the kernels keep
the reference's operand order and are compiled without FMA contraction); the bar stated for
it is 1e-12 relative, checked first.  FP32 fused path: max relative detector-field error
<= 1e-4 (normalised per detector by the max |field| of its trace), emitter dipoles <= 1e-3.
"""
import math
import os
import subprocess
import sys

import numpy as np
import pytest

import omx
from omx import decks
from gpu_harness import (compare_fields, make_pair, point_trace_error, run_both, step_loop, tmz_variant_deck,
                         trace_error)

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))

FP64_TOL = 1e-12
FP32_TOL = 1e-4


def small_cfg1():
    return decks.deck_cfg1(n=32, radius_nm=8.0, npml=6, steps=80)


def small_cfg2():
    return decks.deck_cfg2(nx=240, ny=160, n_emitters=300, npml=8, pitch_nm=120.0, hole_nm=40.0, film_nm=20.0)


def small_cfg3():
    return decks.deck_cfg3(n=64, n_emitters=400, npml=6)


def small_cfg5():
    return decks.deck_cfg5_instance(36, seed=5, npml=6)


def tez_single_group_deck():
    """2D TEz, CPML x / periodic y, Drude disc, radial x-source, a `single` q-group (7x7 kernels)
    and a second `material` group sharing cells (last writer wins across groups)."""
    d = decks._base(2, (96, 80), 8, (3, 2, 1), 2.0, mode=2)
    n = (96, 80)
    g = np.arange(1, 97)
    I, J = np.meshgrid(np.arange(1, 97), np.arange(1, 81), indexing="ij")
    disc = (I - 60.5) ** 2 + (J - 40.5) ** 2 <= 64
    d["media"].append(dict(kind="drude", omegaD=8.0, GammaD=0.3, eps_r=2.0))
    d["voxels"].append(np.stack([decks._cell_nm(I[disc], 96, 2.0), decks._cell_nm(J[disc], 80, 2.0)], axis=1))
    ev, fs = omx.UNITS["ev_to_au"], omx.UNITS["fs_to_au"]
    d["sources"].append(dict(dir="x", j_amp=1.0, w0=2.5 * ev, t0=6 * fs, tau=2 * fs, r0=[-30 * 2 * decks.NM, 0.0],
                             radius=2.2 * d["dr"], t_init=0.0, t_final=1e30, phase=0.3, chirp=0.0))
    rng = np.random.default_rng(9)
    ne = 40
    cells = np.stack([rng.integers(30, 50, ne), rng.integers(20, 60, ne)], axis=1).astype(np.int32)
    par = np.stack([rng.normal(2.5, 0.05, ne) * ev, np.full(ne, 8 * decks.DEBYE), np.full(ne, 500 * fs),
                    np.full(ne, 50 * fs), np.full(ne, 0.6), np.full(ne, 0.8), np.zeros(ne)], axis=1)
    d["groups"].append(dict(group_type=2, model=1, cells=cells, params=par, density=2e-3 / decks.NM ** 3, dt=d["dt"]))
    cells2 = cells[:10] + np.array([1, 0], np.int32)
    par2 = np.stack([np.full(10, 2.4 * ev), np.full(10, 6 * decks.DEBYE), np.full(10, 300 * fs), np.full(10, 40 * fs),
                     np.ones(10), np.zeros(10), np.zeros(10)], axis=1)
    d["groups"].append(dict(group_type=1, model=1, cells=cells2, params=par2, density=1e-3 / decks.NM ** 3,
                            dt=d["dt"]))
    for p in ([20, 20], [70, 60], [50, 11]):
        for f in (1, 2, 6):
            d["detectors"].append(dict(type=1, field=f, idx=np.array([p], np.int32)))
    return d


def one_d_deck():
    """1D CPML, library Ag Drude-Lorentz slab, point source, three-level material group."""
    d = decks._base(1, (400,), 12, (3,), 1.0)
    ev, fs = omx.UNITS["ev_to_au"], omx.UNITS["fs_to_au"]
    d["media"].append(dict(kind="dl_library", material="Ag", eps_r=1.0))
    d["voxels"].append(decks._cell_nm(np.arange(260, 300), 400, 1.0).reshape(-1, 1))
    d["sources"].append(dict(dir="x", j_amp=1.0, w0=3.0 * ev, t0=3 * fs, tau=1 * fs, r0=[-50 * decks.NM], radius=0.0,
                             t_init=0.0, t_final=1e30, phase=0.0, chirp=0.0))
    ne = 5
    cells = np.array([[230], [231], [231], [240], [305]], np.int32)
    par = np.tile([2.9 * ev, 3.1 * ev, 5 * decks.DEBYE, 7 * decks.DEBYE, 800 * fs, 60 * fs, 1.0, 0.0, 0.0], (ne, 1))
    d["groups"].append(dict(group_type=1, model=2, cells=cells, params=par, density=5e-3 / decks.NM ** 3, dt=d["dt"]))
    for k in (100, 250, 280, 330):
        for f in (1, 5):
            d["detectors"].append(dict(type=1, field=f, idx=np.array([[k]], np.int32)))
    return d


def periodic_box_deck(n=(24, 20, 16), boundaries=(2, 2, 2), npml=4, drude=False):
    """3D box (periodic on all axes by default) with a dielectric block (and a Drude block) and a
    radial y-source; line/plane detectors."""
    nx, ny, nz = n
    d = decks._base(3, n, npml, boundaries, 2.0)
    I, J, K = np.meshgrid(np.arange(nx // 3, nx // 3 + 6), np.arange(5, 12), np.arange(nz // 2 - 2, nz // 2 + 2),
                          indexing="ij")
    d["media"].append(dict(kind="dielectric", eps_r=4.0))
    d["voxels"].append(np.stack([decks._cell_nm(I.ravel(), nx, 2.0), decks._cell_nm(J.ravel(), ny, 2.0),
                                 decks._cell_nm(K.ravel(), nz, 2.0)], axis=1))
    if drude:
        I, J, K = np.meshgrid(np.arange(nx // 2 + 4, nx // 2 + 9), np.arange(ny // 2 - 3, ny // 2 + 3),
                              np.arange(nz // 2 - 3, nz // 2 + 2), indexing="ij")
        d["media"].append(dict(kind="drude", omegaD=7.0, GammaD=0.2, eps_r=1.5))
        d["voxels"].append(np.stack([decks._cell_nm(I.ravel(), nx, 2.0), decks._cell_nm(J.ravel(), ny, 2.0),
                                     decks._cell_nm(K.ravel(), nz, 2.0)], axis=1))
    ev, fs = omx.UNITS["ev_to_au"], omx.UNITS["fs_to_au"]
    d["sources"].append(dict(dir="y", j_amp=2.0, w0=2.0 * ev, t0=4 * fs, tau=1.5 * fs, r0=[10 * decks.NM, 0.0, 0.0],
                             radius=1.5 * d["dr"], t_init=0.0, t_final=1e30, phase=0.0, chirp=0.0))
    line = np.array([[i, 3, 4] for i in range(1, nx + 1)], np.int32)
    plane = np.array([[i, j, nz // 2] for j in range(1, ny + 1) for i in range(1, nx + 1)], np.int32)
    for f in range(1, 7):
        d["detectors"].append(dict(type=2, field=f, idx=line))
    d["detectors"].append(dict(type=5, field=3, idx=plane))
    return d


CASES = {
    "cfg1_small": (small_cfg1, 70),
    "cfg2_small": (small_cfg2, 300),
    "cfg3_small": (small_cfg3, 60),
    "cfg5_small": (small_cfg5, 60),
    "tez_single": (tez_single_group_deck, 120),
    "one_d": (one_d_deck, 500),
    "periodic": (periodic_box_deck, 80),
}


@pytest.fixture(scope="module")
def orc_mod(orc):
    return orc


@pytest.mark.parametrize("case", sorted(CASES))
def test_fp64_matches_oracle(orc_mod, case):
    make, steps = CASES[case]
    deck = make()
    gpu, cpu, gg, cg, tc, tg = run_both(orc_mod, deck, steps, "fp64", "calls")
    err = compare_fields(gpu, cpu, deck)
    assert err <= FP64_TOL, err
    assert tg.shape == tc.shape
    assert trace_error(tg, tc) <= FP64_TOL
    # bit-identical is what the exact path delivers
    assert err == 0.0 and np.array_equal(tg, tc), (err, np.max(np.abs(tg - tc)))
    for a, b in zip(gg, cg):
        ga, cb = a.read(), cpu.q_group_read(b)
        for key in ("dipole", "dPt_dt", "E", "rho"):
            assert np.array_equal(ga[key], cb[key]), key


@pytest.mark.parametrize("case", sorted(CASES))
def test_device_loop_matches_calls(orc_mod, case):
    """omx_run (device-side loop, with and without a CUDA graph) equals the per-call API."""
    make, steps = CASES[case]
    deck = make()
    steps = min(steps, 60)
    for graph in (False, True):
        gpu, cpu, gg, cg, tc, tg = run_both(orc_mod, deck, steps, "fp64", "run", use_graph=graph)
        assert compare_fields(gpu, cpu, deck) == 0.0
        assert np.array_equal(tg, tc)


@pytest.mark.parametrize("case", sorted(CASES))
def test_fp32_within_tolerance(orc_mod, case):
    make, steps = CASES[case]
    deck = make()
    gpu, cpu, gg, cg, tc, tg = run_both(orc_mod, deck, steps, "fp32", "run", use_graph=True)
    err = trace_error(tg, tc)
    assert err <= FP32_TOL, err
    for a, b in zip(gg, cg):
        ga, cb = a.read(), cpu.q_group_read(b)
        ref = max(np.max(np.abs(cb["dipole"])), 1e-300)
        assert np.max(np.abs(ga["dipole"] - cb["dipole"])) / ref <= 1e-3


def fused3_deck(n, boundaries, npml=6, src="plane", media_in_cpml=True, emitters=True):
    """3D scene for the single-pass FP32 step: a dielectric block, a Drude block and a
    Drude-Lorentz gold block (one of them reaching into the low-x CPML slab when media_in_cpml),
    a plane Ex sheet (folded into the pass) or a radial y-source plus a plane (added after the
    pass), a three-level `material` group, point detectors on E and H near the tile edges."""
    nx, ny, nz = n
    d = decks._base(3, n, npml, boundaries, 2.0)
    ev, fs = omx.UNITS["ev_to_au"], omx.UNITS["fs_to_au"]

    def block(x0, x1, y0, y1, z0, z1):
        I, J, K = np.meshgrid(np.arange(x0, x1), np.arange(y0, y1), np.arange(z0, z1), indexing="ij")
        return np.stack([decks._cell_nm(I.ravel(), nx, 2.0), decks._cell_nm(J.ravel(), ny, 2.0),
                         decks._cell_nm(K.ravel(), nz, 2.0)], axis=1)

    zc = nz // 2
    d["media"].append(dict(kind="dielectric", eps_r=4.0))
    d["voxels"].append(block(nx // 3, nx // 3 + 5, 3, 9, zc - 2, zc + 2))
    d["media"].append(dict(kind="drude", omegaD=7.0, GammaD=0.2, eps_r=1.5))
    d["voxels"].append(block(nx // 2 + 2, nx // 2 + 7, ny // 2 - 3, ny // 2 + 3, zc - 3, zc + 2))
    d["media"].append(dict(decks.GOLD_DL))
    x0 = 2 if media_in_cpml else npml + 2
    d["voxels"].append(block(x0, x0 + 6, ny - 12, ny - 5, zc - 1, zc + 3))
    tau = 1.5 * fs
    # the Ex sheet below the media (a sheet added after the pass must not cross a dispersive cell)
    d["plane_sources"].append(dict(comp=1, plane_axis=3, plane_index=max(2, min(npml + 3, zc - 5)), j_amp=3.0,
                                   w0=2.2 * ev, t0=3 * tau,
                                   tau=tau, t_init=0.0, t_final=1e30, phase=0.0, chirp=0.0))
    if src == "both":
        d["sources"].append(dict(dir="y", j_amp=2.0, w0=2.0 * ev, t0=4 * fs, tau=1.5 * fs,
                                 r0=[-6 * 2.0 * decks.NM, 4 * 2.0 * decks.NM, 0.0], radius=1.5 * d["dr"],
                                 t_init=0.0, t_final=1e30, phase=0.0, chirp=0.0))
    if emitters:
        rng = np.random.default_rng(sum(n))
        ne = 40
        cells = np.stack([rng.integers(npml + 2, nx - npml - 1, ne), rng.integers(npml + 2, ny - npml - 1, ne),
                          rng.integers(zc + 2, max(zc + 3, nz - npml - 1), ne)], axis=1).astype(np.int32)
        u = rng.normal(size=(ne, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        par = np.concatenate([np.stack([rng.normal(2.1, 0.03, ne) * ev, rng.normal(2.3, 0.03, ne) * ev,
                                        np.full(ne, 6 * decks.DEBYE), np.full(ne, 7 * decks.DEBYE),
                                        np.full(ne, 500 * fs), np.full(ne, 60 * fs)], axis=1), u], axis=1)
        d["groups"].append(dict(group_type=1, model=2, cells=cells, params=par, density=3e-3 / decks.NM ** 3,
                                dt=d["dt"]))
    # points on tile edges (x = 32 | 33, y = 8 | 9 | 16, z = 64 | 65 where a plane chunk ends), in
    # the gold block and near the k = 1 / nz planes, kept out of the CPML corners and off PEC walls,
    # where the field is absorbed to values whose FP32 relative error says nothing
    lo = [npml + 2 if b == 3 else 2 for b in boundaries]
    hi = [m - (npml + 1 if b == 3 else 2) for m, b in zip(n, boundaries)]
    pts = ([32, 8, zc], [33, 9, zc + 1], [32, 16, zc - 2], [nx // 2, ny // 2, lo[2]], [nx // 2, ny // 2, hi[2]],
           [x0 + 2, ny - 8, zc + 1], [nx // 2 + 4, ny // 2, zc], [nx // 2, 9, 64], [nx // 2 - 1, 8, 65])
    for p in pts:
        p = [min(max(v, l), h) for v, l, h in zip(p, lo, hi)]
        for f in (1, 2, 3, 4, 6):
            d["detectors"].append(dict(type=1, field=f, idx=np.array([p], np.int32)))
    return d


def _fused3_ran(g, deck):
    """True when the grid steps with one pass per step (no H-only launches)."""
    g.profile(True)
    g.run(10_000, 2, deck["n_skip"], 0, use_graph=False)
    g.synchronize()
    _, nh = g.profile_query(omx.KC_H)
    _, ne = g.profile_query(omx.KC_E)
    g.profile(False)
    return nh == 0 and ne == 2


@pytest.mark.parametrize("n,boundaries,src,steps", [
    ((40, 36, 28), (3, 3, 3), "plane", 90),    # CPML on every face, partial tiles in x and y, DL in the CPML
    ((64, 24, 20), (3, 3, 2), "plane", 90),    # periodic z: plane 0 is the image of plane nz
    ((33, 17, 19), (1, 1, 1), "both", 80),     # PEC box, odd sizes, a radial source after the pass
    ((48, 40, 70), (3, 1, 3), "plane", 100),   # several planes chunks along z
    ((62, 20, 18), (1, 1, 3), "plane", 60),    # PEC x: the last tile's lean planes reach the row's end
])
def test_fp32_fused3d(orc_mod, n, boundaries, src, steps):
    """The FP32 single-pass 3D step (k_fused3_tma, the default 3D FP32 form when x and y are not
    periodic): detector traces and fields within the FP32 bar of the FP64 oracle, through the
    device loop and through the per-call sequence (omx_step_H deferred into the fused pass).

    The detector bar is relative to the field at each detector's point (point_trace_error): the
    scene puts E and H detectors of every component at each point, and some components vanish
    there by symmetry (Hx beside the Ex sheet reaches 1e-5 of the point's H), so their own
    maximum is no scale for an FP32 rounding error -- the plain two-pass FP32 step shows the same
    per-component figure (2.7e-3 at such a detector) as this pass (3.0e-3)."""
    deck = fused3_deck(n, boundaries, src=src)
    for mode in ("run", "calls"):
        gpu, cpu, gg, cg, tc, tg = run_both(orc_mod, deck, steps, "fp32", mode, use_graph=True)
        assert np.max(np.abs(tc)) > 0
        err = point_trace_error(tg, tc, deck)
        assert err <= FP32_TOL, (mode, err)
        assert compare_fields(gpu, cpu, deck) <= 10 * FP32_TOL
        for a, b in zip(gg, cg):
            ga, cb = a.read(), cpu.q_group_read(b)
            ref = max(np.max(np.abs(cb["dipole"])), 1e-300)
            assert np.max(np.abs(ga["dipole"] - cb["dipole"])) / ref <= 1e-3
        assert _fused3_ran(gpu, deck)
        gpu.kill()


def test_fused3d_shapes_bit_identical():
    """Every tile shape of the fused 3D pass (8 or 16 rows, any planes per block) computes each
    cell with the same operations: the halo H a block recomputes equals its owner's bit for bit,
    so fields, records and emitter state agree bit for bit across shapes."""
    deck = fused3_deck((72, 44, 50), (3, 3, 3), src="plane")
    out = []
    for shape in (8064, 8016, 16032, 8007, 16128):
        g = omx.TMxll(3, deck["grid_Ndims"], deck["npml"], deck["boundaries"], deck["dt"], deck["dr"],
                      precision="fp32")
        groups = decks.apply_deck(g, deck, omx, decks.media_map(deck, omx.media_map_from_voxels))
        for det in deck["detectors"]:
            g.add_detector(det["type"], det["field"], det["idx"])
        g.set_launch_shape(shape)
        g.run(1, 60, deck["n_skip"], 1)
        _, tr = g.drain_detectors()
        st = groups[0].read()
        out.append((tr, [g.read_field(f) for f in range(1, 7)], st["rho"]))
        assert _fused3_ran(g, deck)
        g.kill()
    t0, f0, r0 = out[0]
    assert np.max(np.abs(t0)) > 0
    for t, f, r in out[1:]:
        assert np.array_equal(t, t0) and np.array_equal(r, r0)
        for a, b in zip(f, f0):
            assert np.array_equal(a, b)


def test_cfg1_full_size_fp64_bit_exact(orc_mod):
    """The plain 3D configuration at its full size and length: 128^3, dr 2 nm, 10-cell CPML on
    every face, the Drude-Lorentz gold sphere (r 20 nm), the 2.2 eV plane-wave sheet, 16 point
    detectors sampled every step, 4000 steps (the oracle takes about a minute on 16 cores).  The
    FP64 GPU path equals the oracle bit for bit: every detector sample and every field word."""
    deck = decks.deck_cfg1()
    assert deck["grid_Ndims"] == [128, 128, 128] and deck["steps"] == 4000
    gpu, cpu, gg, cg, tc, tg = run_both(orc_mod, deck, deck["steps"], "fp64", "run", use_graph=True)
    assert tg.shape == tc.shape == (4000, 16)
    assert np.max(np.abs(tc)) > 0
    assert np.array_equal(tg, tc), trace_error(tg, tc)
    assert compare_fields(gpu, cpu, deck) == 0.0
    gpu.kill()


def test_cfg2_full_size_fp64_prefix_bit_exact(orc_mod):
    """The 2D TMz configuration at its full size (4096^2, periodic x / CPML y, perforated Drude
    silver film, 1e4 two-level emitters, 16 point detectors): the first 200 steps of the FP64
    GPU path equal the oracle bit for bit (fields, detector samples, density matrices)."""
    deck = decks.deck_cfg2()
    assert deck["grid_Ndims"] == [4096, 4096] and len(deck["groups"][0]["cells"]) == 10000
    steps = 200
    gpu, cpu, gg, cg, tc, tg = run_both(orc_mod, deck, steps, "fp64", "run", use_graph=True)
    assert np.max(np.abs(cpu.read_field(omx.EZ))) > 0      # the pulse is on the grid
    assert np.array_equal(tg, tc), trace_error(tg, tc)
    assert compare_fields(gpu, cpu, deck) == 0.0
    ga, cb = gg[0].read(), cpu.q_group_read(cg[0])
    for key in ("dipole", "rho", "E"):
        assert np.array_equal(ga[key], cb[key]), key
    gpu.kill()


def test_long_run_fp64_cfg1_shape(orc_mod):
    """A longer plain 3D run (Au sphere, plane wave, CPML) keeps bit parity over 400 steps."""
    deck = decks.deck_cfg1(n=40, radius_nm=10.0, npml=8)
    gpu, cpu, gg, cg, tc, tg = run_both(orc_mod, deck, 400, "fp64", "run", use_graph=True)
    assert compare_fields(gpu, cpu, deck) == 0.0
    assert np.array_equal(tg, tc)


def test_media_after_start_is_rejected(orc_mod):
    deck = small_cfg1()
    gpu = omx.TMxll(3, deck["grid_Ndims"], deck["npml"], deck["boundaries"], deck["dt"], deck["dr"])
    gpu.td_propagate_H_field()
    with pytest.raises(omx.OMXError):
        gpu.set_media([omx.medium_dielectric(2.0)], np.zeros((32, 32, 32, 3), np.int32))
    with pytest.raises(omx.OMXError):
        omx.TMxll(3, (40, 40, 40), 25, (3, 3, 3), deck["dt"], deck["dr"])   # two CPML slabs do not fit


@pytest.mark.parametrize("shape,bx,by,src,steps", [
    ((128, 96), 2, 3, "plane", 301),     # periodic x, CPML y (the benchmark's boundaries), odd steps
    ((96, 64), 2, 2, "radial", 240),     # periodic x and y
    ((128, 100), 3, 3, "plane", 250),    # CPML on both axes
    ((64, 72), 1, 1, "radial", 200),     # closed (PEC) box
    ((102, 80), 2, 3, "plane", 200),     # width not a multiple of 4: the unfused FP32 kernels
    # wide grids (enough steps for the wave to reach the scatterers, so that every component
    # carries a field well inside the FP32 range)
    ((1540, 300), 2, 3, "plane", 260),   # 4 column strips, the last with one active thread
    ((1028, 420), 3, 3, "radial", 260),  # x CPML across strips; blocks span strip boundaries
])
def test_fp32_fused_tmz_variants(orc_mod, shape, bx, by, src, steps):
    deck = tmz_variant_deck(shape[0], shape[1], bx, by, src=src)
    gpu, cpu, gg, cg, tc, tg = run_both(orc_mod, deck, steps, "fp32", "run", use_graph=True)
    assert trace_error(tg, tc) <= FP32_TOL
    assert compare_fields(gpu, cpu, deck) <= 10 * FP32_TOL
    ga, cb = gg[0].read(), cpu.q_group_read(cg[0])
    # dipoles below 1e-30 a.u. (emitters the wave has not reached) count as zero
    assert np.max(np.abs(ga["dipole"] - cb["dipole"])) / max(np.max(np.abs(cb["dipole"])), 1e-30) <= 1e-3
    # the per-call API on the same FP32 context type agrees with the device loop
    gpu2, cpu2, gg2, cg2, tc2, tg2 = run_both(orc_mod, deck, steps, "fp32", "calls")
    assert trace_error(tg2, tc) <= FP32_TOL


FORMS = ("regs", "tma4", "tma5", "tma6", "tma8", "ws4", "ws5", "ws6", "ws4x2", "ws5x2", "ws4w8", "ws5w8", "rt4", "rt6")


@pytest.mark.parametrize("shape,bx,by,src,steps", [
    ((2052, 900), 2, 3, "plane", 80),    # several rows per block, segments crossing strips
    ((1028, 260), 3, 3, "radial", 120),  # x CPML (the other kernel instance)
    ((96, 64), 2, 2, "radial", 41),      # periodic x and y, one row per block
])
def test_fused_forms_bit_identical(tmp_path, shape, bx, by, src, steps):
    """Every form of the fused TMz kernel (register prefetch, bulk copies into rings of 4-8
    slots, with or without a dedicated copy warp, one or two 4-cell chunks per thread) performs
    the same arithmetic on the same words: fields and detector traces agree bit for bit.  Each form runs in its own process (the form is chosen once per process)."""
    out = {}
    for form in FORMS:
        f = tmp_path / f"{form}.npz"
        env = dict(os.environ, OMX_FUSED_KERNEL=form)
        r = subprocess.run([sys.executable, os.path.join(HERE, "fused_form_child.py"), str(shape[0]), str(shape[1]),
                            str(bx), str(by), src, str(steps), str(f)], env=env, capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        out[form] = np.load(f)
    base = out[FORMS[0]]
    assert np.max(np.abs(base["f3"])) > 0.0
    for form in FORMS[1:]:
        for key in base.files:
            assert np.array_equal(out[form][key], base[key]), (form, key)


@pytest.mark.parametrize("case,precision", [("cfg1_small", "fp64"), ("cfg3_small", "fp32"), ("tez_single", "fp64")])
def test_autotune_leaves_no_trace(orc_mod, case, precision):
    """The autotuner times its candidates on the zero initial fields: afterwards the run gives
    the same result as without it (bit-identical for FP64, within the FP32 bar otherwise)."""
    make, steps = CASES[case]
    deck = make()
    n = min(steps, 60)
    gpu, cpu, gg, cg, tc, tg = run_both(orc_mod, deck, n, precision, "run", autotune=True)
    if precision == "fp64":
        assert np.array_equal(tg, tc)
    else:
        assert trace_error(tg, tc) <= FP32_TOL
    with pytest.raises(omx.OMXError):
        gpu.autotune(reps=1)                  # after the first step: refused


def test_autotune_fused_tmz(orc_mod):
    deck = tmz_variant_deck(256, 96, 2, 3, src="plane")
    gpu, cpu, gg, cg, tc, tg = run_both(orc_mod, deck, 120, "fp32", "run", autotune=True)
    assert trace_error(tg, tc) <= FP32_TOL


def test_one_step_calls_with_async_drain_equal_one_run():
    """A host that drives the fused path one omx_run call per step leaves each step's side-stream
    work running into the next call, and drains every step asynchronously (tickets collected one
    step late); fields, detector records and emitter state equal a single multi-step run bit for
    bit, also with unrelated entry points (a field read) between the calls."""
    deck = tmz_variant_deck(256, 64, 2, 3, src="plane")
    n = 37
    out = []
    for mode in ("one_run", "per_step"):
        g = omx.TMxll(2, deck["grid_Ndims"], deck["npml"], deck["boundaries"], deck["dt"], deck["dr"], mode=omx.TMZ,
                      precision="fp32")
        groups = decks.apply_deck(g, deck, omx, decks.media_map(deck, omx.media_map_from_voxels))
        for det in deck["detectors"]:
            g.add_detector(det["type"], det["field"], det["idx"])
        if mode == "one_run":
            g.run(1, n, deck["n_skip"], 1)
            times, tr = g.drain_detectors()
        else:
            tl, vl = [], []
            pending = None
            for tt in range(1, n + 1):
                g.run(tt, 1, deck["n_skip"], 1)
                if tt == 17:
                    g.read_field(3)
                t = g.drain_async()
                if pending is not None:
                    a, b = g.collect(pending)
                    tl.append(a)
                    vl.append(b)
                pending = t
            a, b = g.collect(pending)
            tl.append(a)
            vl.append(b)
            times, tr = np.concatenate(tl), np.concatenate(vl)
        st = groups[0].read()
        out.append((times, tr, [g.read_field(f) for f in (3, 4, 5)], st["rho"], st["dipole"]))
        g.kill()
    (s0, t0, f0, r0, d0), (s1, t1, f1, r1, d1) = out
    assert len(s0) == n and np.max(np.abs(t0)) > 0 and np.max(np.abs(d0)) > 0
    assert np.array_equal(s0, s1) and np.array_equal(t0, t1)
    assert np.array_equal(r0, r1) and np.array_equal(d0, d1)
    for a, b in zip(f0, f1):
        assert np.array_equal(a, b)


def _tmz_context(deck):
    g = omx.TMxll(2, deck["grid_Ndims"], deck["npml"], deck["boundaries"], deck["dt"], deck["dr"], mode=omx.TMZ,
                  precision="fp32")
    groups = decks.apply_deck(g, deck, omx, decks.media_map(deck, omx.media_map_from_voxels))
    for det in deck["detectors"]:
        g.add_detector(det["type"], det["field"], det["idx"])
    return g, groups


def test_per_call_sequence_runs_the_fused_pass():
    """The reference's per-step calls (omx_step_H, omx_source_interactions, omx_step_E,
    omx_qgroup_step, omx_detectors_record) on the FP32 TMz path defer the H half into the fused
    pass of omx_step_E: bit-identical to omx_run.  An entry point between the H and E calls (a
    field read) runs the deferred H half unfused; that run agrees with the fused one to FP32
    rounding."""
    deck = tmz_variant_deck(256, 64, 2, 3, src="plane")
    n = 41
    out = []
    for mode in ("run", "calls", "calls_flushed"):
        g, groups = _tmz_context(deck)
        if mode == "run":
            g.run(1, n, deck["n_skip"], deck["t_det_print"])
        else:
            class Target:
                def __getattr__(self, k):
                    return getattr(g, k)

                def td_propagate_H_field(self):
                    g.td_propagate_H_field()
                    if mode == "calls_flushed":
                        g.read_field(4)

            step_loop(Target(), deck, groups, 1, n, {"tq_old": 0, "t_skip": 0.0},
                      sample=lambda t: g.write_detectors_outputs(t))
        _, tr = g.drain_detectors()
        st = groups[0].read()
        out.append((tr, [g.read_field(f) for f in (3, 4, 5)], st["rho"], st["dipole"]))
        g.kill()
    (t0, f0, r0, d0), (t1, f1, r1, d1), (t2, f2, r2, d2) = out
    assert np.max(np.abs(t0)) > 0 and np.max(np.abs(d0)) > 0
    assert np.array_equal(t0, t1) and np.array_equal(r0, r1) and np.array_equal(d0, d1)
    for a, b in zip(f0, f1):
        assert np.array_equal(a, b)
    assert not np.array_equal(t0, t2)          # the flushed run did take the unfused path
    assert trace_error(t2, t0) <= FP32_TOL


@pytest.mark.parametrize("case,precision,form", [("cfg1_small", "fp32", omx.STEP_TWO_PASS),
                                                 ("cfg3_small", "fp32", omx.STEP_TWO_PASS),
                                                 ("cfg3_small", "fp64", None),
                                                 ("cfg1_small", "fp32", None), ("cfg3_small", "fp32", None)])
def test_two_pass_one_step_calls_equal_one_run(case, precision, form):
    """A 3D grid driven one omx_run call per step leaves each step's sampling and emitter work
    running next to the next call's first pass (the two-pass path's H pass, or the fused pass),
    with asynchronous drains collected two steps late; records, fields and emitter state equal a
    single multi-step run bit for bit."""
    deck = CASES[case][0]()
    n = 23
    out = []
    for mode in ("one_run", "per_step"):
        g = omx.TMxll(3, deck["grid_Ndims"], deck["npml"], deck["boundaries"], deck["dt"], deck["dr"],
                      precision=precision)
        if precision == "fp32" and form is not None:
            g.set_step_form(form)
        mm = decks.media_map(deck, omx.media_map_from_voxels) if deck["voxels"] else None
        groups = decks.apply_deck(g, deck, omx, mm)
        for det in deck["detectors"]:
            g.add_detector(det["type"], det["field"], det["idx"])
        if mode == "one_run":
            g.run(1, n, deck["n_skip"], 1)
            times, tr = g.drain_detectors()
        else:
            tl, vl, pending = [], [], []
            for tt in range(1, n + 1):
                g.run(tt, 1, deck["n_skip"], 1)
                if tt == 11:
                    g.read_field(1)
                pending.append(g.drain_async())
                if len(pending) > 2:
                    a, b = g.collect(pending.pop(0))
                    tl.append(a)
                    vl.append(b)
            while pending:
                a, b = g.collect(pending.pop(0))
                tl.append(a)
                vl.append(b)
            times, tr = np.concatenate(tl), np.concatenate(vl)
        st = groups[0].read() if groups else None
        out.append((times, tr, [g.read_field(f) for f in (1, 2, 3, 4, 5, 6)], st))
        g.kill()
    (s0, t0, f0, g0), (s1, t1, f1, g1) = out
    assert len(s0) == n and np.max(np.abs(t0)) > 0
    assert np.array_equal(s0, s1) and np.array_equal(t0, t1)
    for a, b in zip(f0, f1):
        assert np.array_equal(a, b)
    if g0 is not None:
        assert np.array_equal(g0["rho"], g1["rho"]) and np.array_equal(g0["dipole"], g1["dipole"])


def test_async_drain_ring_limits():
    deck = tmz_variant_deck(128, 48, 2, 2, src="plane")
    g = omx.TMxll(2, deck["grid_Ndims"], deck["npml"], deck["boundaries"], deck["dt"], deck["dr"], mode=omx.TMZ,
                  precision="fp32")
    decks.apply_deck(g, deck, omx, decks.media_map(deck, omx.media_map_from_voxels))
    for det in deck["detectors"]:
        g.add_detector(det["type"], det["field"], det["idx"])
    tickets = []
    for tt in range(1, 5):
        g.run(tt, 1, deck["n_skip"], 1)
        tickets.append(g.drain_async())
    with pytest.raises(omx.OMXError):
        g.drain_async()                       # all four slots hold uncollected tickets
    with pytest.raises(omx.OMXError):
        g.collect(tickets[0] + 100)           # unknown ticket
    times, _ = g.collect(tickets[0])
    assert len(times) == 1
    with pytest.raises(omx.OMXError):
        g.collect(tickets[0])                 # already collected
    g.run(5, 3, deck["n_skip"], 1)
    t5 = g.drain_async()
    with pytest.raises(omx.OMXError):
        g.collect(t5, max_records=2)          # three records do not fit
    for t in tickets[1:]:
        assert len(g.collect(t)[0]) == 1
    g.kill()


@pytest.mark.parametrize("steps", [61, 80])
def test_fused_graph_overlap_equals_sequential(steps):
    """In a graph the fused path runs step s's sampling and emitter work on a side stream next to
    step s+1's fused pass; the result equals the sequential launch order bit for bit (fields,
    detector records, emitter state).  61 steps: 16-step graphs, 2-step graphs and a 1-step graph."""
    deck = tmz_variant_deck(256, 64, 2, 3, src="plane")
    out = []
    for graph in (False, True):
        g = omx.TMxll(2, deck["grid_Ndims"], deck["npml"], deck["boundaries"], deck["dt"], deck["dr"], mode=omx.TMZ,
                      precision="fp32")
        groups = decks.apply_deck(g, deck, omx, decks.media_map(deck, omx.media_map_from_voxels))
        for det in deck["detectors"]:
            g.add_detector(det["type"], det["field"], det["idx"])
        g.run(1, 20, deck["n_skip"], deck["t_det_print"], use_graph=graph)
        g.run(21, steps, deck["n_skip"], deck["t_det_print"], use_graph=graph)
        _, tr = g.drain_detectors()
        st = groups[0].read()
        out.append((tr, [g.read_field(f) for f in (3, 4, 5)], st["rho"], st["dipole"]))
        g.kill()
    (t0, f0, r0, d0), (t1, f1, r1, d1) = out
    assert np.max(np.abs(d0)) > 0 and np.max(np.abs(t0)) > 0
    assert np.array_equal(t0, t1) and np.array_equal(r0, r1) and np.array_equal(d0, d1)
    for a, b in zip(f0, f1):
        assert np.array_equal(a, b)
