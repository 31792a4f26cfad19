"""Batched multi-grid runs (omx_batch_*): several 3D instances of the inverse-design sweep advance
together -- FP32 grids that step with one fused pass in one k_fused3_batch launch per step (or the
pass split by plane form), the others through one persistent launch per half-step pass; every grid must equal its own solo run
bit for bit (same arithmetic, same per-grid order), with and without the graph and after the
batch autotuner.  Calls go through the C-ABI."""
import numpy as np
import pytest

import omx
from omx import decks

pytestmark = pytest.mark.gpu

SIZES = (36, 44, 29, 52)     # uneven sides, none a multiple of the 32-cell tile width


def build(n, seed, precision):
    d = decks.deck_cfg5_instance(n, seed=seed, npml=6)
    g = omx.TMxll(3, d["grid_Ndims"], d["npml"], d["boundaries"], d["dt"], d["dr"], precision=precision)
    decks.apply_deck(g, d, omx, decks.media_map(d, omx.media_map_from_voxels))
    for det in d["detectors"]:
        g.add_detector(det["type"], det["field"], det["idx"])
    return d, g


def fields(g):
    return [g.read_field(f) for f in (1, 2, 3, 4, 5, 6)]


@pytest.mark.parametrize("precision,form", [("fp32", omx.STEP_DEFAULT), ("fp32", omx.STEP_TWO_PASS),
                                            ("fp64", omx.STEP_DEFAULT)])
@pytest.mark.parametrize("use_graph,autotune", [(True, False), (False, False), (True, True)])
def test_batch_equals_solo_runs(precision, form, use_graph, autotune):
    steps = 70
    solo, batch = [], []
    for k, n in enumerate(SIZES):
        d, g = build(n, 100 + k, precision)
        g.set_step_form(form)                 # the batch runs its members' arithmetic
        g.run(1, steps, d["n_skip"], d["t_det_print"], use_graph=True)
        solo.append((fields(g), g.drain_detectors()[1]))
        g.kill()
        batch.append(build(n, 100 + k, precision))
        batch[-1][1].set_step_form(form)
    b = omx.Batch([g for _, g in batch])
    if autotune:
        fused = precision == "fp32" and form == omx.STEP_DEFAULT
        choice = b.autotune(reps=2)
        if fused:
            # split grids x 1000000 + (ring depth x 100 + tile rows) x 1000 + planes per block
            form = choice // 1000 % 1000
            assert 0 <= choice // 1000000 <= len(SIZES) and form % 100 in (8, 16) and form // 100 in (0, 6, 8)
            assert choice % 1000 in (16, 32, 64, 128)
        else:
            assert choice in (4, 8, 16, 32)
    d0 = batch[0][0]
    b.run(1, 30, d0["n_skip"], d0["t_det_print"], use_graph=use_graph)   # two calls: the stepping state carries over
    b.run(31, steps - 30, d0["n_skip"], d0["t_det_print"], use_graph=use_graph)
    assert b.launch_count() > 0
    for (d, g), (f_solo, tr_solo) in zip(batch, solo):
        tr = g.drain_detectors()[1]
        assert tr.shape == tr_solo.shape and np.max(np.abs(tr_solo)) > 0
        assert np.array_equal(tr, tr_solo)
        for a, s in zip(fields(g), f_solo):
            assert np.array_equal(a, s)
    b.kill()
    for _, g in batch:
        g.kill()


@pytest.mark.parametrize("shape", [8064, 1016032, 3608016])
def test_fused_batch_shapes_equal_solo_runs(shape):
    """FP32 fused batch in a set launch shape: every grid in one k_fused3_batch launch (8064), the
    largest grid in the pass split by plane form and the others in one launch (1016032: tile
    32 x 16, 32 planes per lean run), or all three split (3608016: ring of 6, tile 32 x 8, 16
    planes), where the 96^3 grid has lean runs clear of its CPML slabs and the small grids are
    general runs only; every grid equals its solo run bit for bit."""
    sizes, steps = (96, 36, 29), 50
    solo, batch = [], []
    for k, n in enumerate(sizes):
        d, g = build(n, 500 + k, "fp32")
        g.run(1, steps, d["n_skip"], d["t_det_print"], use_graph=True)
        solo.append((fields(g), g.drain_detectors()[1]))
        g.kill()
        batch.append(build(n, 500 + k, "fp32"))
    b = omx.Batch([g for _, g in batch])
    for bad in (4008064, 8, 16000, 8200):    # 4 of 3 grids split, a two-pass depth, 0 planes, 200 planes
        with pytest.raises(omx.OMXError):
            b.set_launch_shape(bad)
    b.set_launch_shape(shape)
    d0 = batch[0][0]
    b.run(1, 20, d0["n_skip"], d0["t_det_print"], use_graph=False)
    b.run(21, steps - 20, d0["n_skip"], d0["t_det_print"], use_graph=True)
    for (d, g), (f_solo, tr_solo) in zip(batch, solo):
        tr = g.drain_detectors()[1]
        assert tr.shape == tr_solo.shape and np.array_equal(tr, tr_solo)
        assert max(np.max(np.abs(f)) for f in f_solo) > 0     # the source has driven every grid
        for a, s_ in zip(fields(g), f_solo):
            assert np.array_equal(a, s_)
    b.kill()
    for _, g in batch:
        g.kill()


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_batch_with_a_grid_that_launches_alone(precision):
    """Two-pass batch: a grid of at least 8 tiles per SM (160^3 here) keeps its own H / E launches
    inside the batched step while the small grids share the persistent passes; every grid still
    equals its solo run bit for bit."""
    sizes, steps = (160, 36, 29), 40
    solo, batch = [], []
    for k, n in enumerate(sizes):
        d, g = build(n, 300 + k, precision)
        g.set_step_form(omx.STEP_TWO_PASS)
        g.run(1, steps, d["n_skip"], d["t_det_print"], use_graph=True)
        solo.append((fields(g), g.drain_detectors()[1]))
        g.kill()
        batch.append(build(n, 300 + k, precision))
        batch[-1][1].set_step_form(omx.STEP_TWO_PASS)
    b = omx.Batch([g for _, g in batch])
    d0 = batch[0][0]
    b.run(1, steps, d0["n_skip"], d0["t_det_print"], use_graph=True)
    for (d, g), (f_solo, tr_solo) in zip(batch, solo):
        tr = g.drain_detectors()[1]
        assert tr.shape == tr_solo.shape and np.array_equal(tr, tr_solo)
        assert max(np.max(np.abs(f)) for f in f_solo) > 0     # the source has driven every grid
        for a, s_ in zip(fields(g), f_solo):
            assert np.array_equal(a, s_)
    b.kill()
    for _, g in batch:
        g.kill()


def test_batch_rejects_bad_members():
    d, g3 = build(32, 1, "fp32")
    _, g64 = build(32, 2, "fp64")
    d2 = decks.deck_cfg2(nx=64, ny=48, n_emitters=4, npml=6, pitch_nm=60.0, hole_nm=20.0, film_nm=10.0)
    g2 = omx.TMxll(2, d2["grid_Ndims"], d2["npml"], d2["boundaries"], d2["dt"], d2["dr"], mode=omx.TMZ)
    for members in ([g3, g64], [g3, g3], [g3, g2]):
        with pytest.raises(omx.OMXError):
            omx.Batch(members)
    g3.run(1, 2, 1, 0)
    b = omx.Batch([g3])
    with pytest.raises(omx.OMXError):
        b.autotune(reps=1)                    # after a first step: refused
    b.kill()
    for g in (g3, g64, g2):
        g.kill()
