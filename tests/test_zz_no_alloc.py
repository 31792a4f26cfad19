"""The emitter step that allocates nothing (omx_emitter_step_noalloc).

It serves hosts that cannot call cudaMalloc in their time loop: they own all device memory
through their own pool or device arrays, and an allocation there would synchronise the whole
device.  For the same inputs it must give what the context API's q-group step gives, on two
calls in a row (the second call finds the shared scratch array holding the first call's values).

The file sorts last so that a run that stops at the first failure has run every other test
before it.  Device buffers come from torch (plumbing only); the call goes through the C-ABI.
"""
import ctypes as C

import numpy as np
import pytest

import omx
from omx import decks

pytestmark = pytest.mark.gpu

TOL = 1e-12   # the FP64 tolerance of the parity tests (the path is expected to be bit-identical)
MAX_EMITTERS = 65536


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _scene_tmz():
    """2D TMz, two-level emitters: the current has the z component only."""
    deck = decks.deck_cfg2(nx=128, ny=96, n_emitters=80, npml=8, pitch_nm=100.0, hole_nm=30.0, film_nm=20.0)
    return deck, omx.TWO_LEVEL, (2, 2)


def _scene_3d():
    """3D, three-level emitters with seeded random orientations: all three current components."""
    deck = decks.deck_cfg3(n=48, n_emitters=150, npml=6)
    p = deck["groups"][0]["params"]
    u = np.random.default_rng(7).normal(size=(len(p), 3))
    p[:, 6:9] = u / np.linalg.norm(u, axis=1, keepdims=True)
    return deck, omx.THREE_LEVEL, (0, 2)


def _build(deck):
    g = omx.TMxll(deck["dimensions"], deck["grid_Ndims"], deck["npml"], deck["boundaries"], deck["dt"], deck["dr"],
                  mode=deck["mode"], precision="fp64")
    groups = decks.apply_deck(g, deck, omx, decks.media_map(deck, omx.media_map_from_voxels))
    return g, groups[0]


def _advance(g, deck, group, state, tt):
    time = deck["dt"] * (tt - 0.5)
    state["t_skip"] = time                     # n_skip = 1: every step is a quantum step
    g.td_propagate_H_field()
    g.source_interactions(time)
    g.td_propagate_E_field(time, state["t_skip"])
    g.q_group_step(group, tt)


@pytest.mark.parametrize("scene", [_scene_tmz, _scene_3d], ids=["tmz_two_level", "3d_three_level"])
def test_noalloc_emitter_step_matches_qgroup_step(scene):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    L = omx.lib()
    deck, model, (c0, c1) = scene()
    assert deck["n_skip"] == 1
    g, group = _build(deck)
    gd = deck["groups"][0]
    n = len(gd["cells"])
    # current points of a `material` group: the distinct emitter cells; the last emitter in a
    # cell writes it (interactions_mod.f90:1181-1190).  Two extra points that no emitter of this
    # call writes (winner -1, and an index past the call's emitters) must keep their current.
    keys = [tuple(c) for c in gd["cells"]]
    uniq = sorted(set(keys))
    slot = {k: p for p, k in enumerate(uniq)}
    winner = np.full(len(uniq), -1, np.int32)
    for e, k in enumerate(keys):
        winner[slot[k]] = e
    nreal = len(uniq)
    winner = np.concatenate([winner, np.array([-1, n + 5], np.int32)])
    npnt = len(winner)
    wk = np.full(npnt, gd["density"])
    dt = gd["dt"]

    state = {"t_skip": 0.0}
    for tt in range(1, 60):
        _advance(g, deck, group, state, tt)
    prev = group.read()
    J_prev = np.zeros((3, npnt))
    for c in range(c0, c1 + 1):
        J_prev[c, :nreal] = wk[:nreal] * prev["dPt_dt"][winner[:nreal], c]
        J_prev[c, nreal:] = [0.25 + c, -1.5 - c]     # arbitrary currents the call must keep

    dev = torch.device("cuda:0")
    t = lambda a, dtype=torch.float64: torch.tensor(np.ascontiguousarray(a), dtype=dtype, device=dev)
    E_d = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    par_d = t(gd["params"])
    rho_d = t(prev["rho"])
    dip_d = t(prev["dipole"])
    win_d = t(winner, torch.int32)
    wk_d = t(wk)
    J_d = t(J_prev)
    Jo_d = torch.zeros_like(J_d)
    dJ_d = torch.zeros_like(J_d)
    stream = torch.cuda.current_stream(dev).cuda_stream

    def call_noalloc(s):
        return L.omx_emitter_step_noalloc(model, n, E_d.data_ptr(), par_d.data_ptr(), rho_d.data_ptr(),
                                          dip_d.data_ptr(), npnt, win_d.data_ptr(), wk_d.data_ptr(), J_d.data_ptr(),
                                          Jo_d.data_ptr(), dJ_d.data_ptr(), c0, c1, dt, C.c_void_p(s))

    # steps 60, 61: direct calls; step 62: the call captured in a CUDA graph (it allocates
    # nothing, so it captures) with its input E written after the capture, then one replay
    for call, tt in enumerate((60, 61, 62)):
        _advance(g, deck, group, state, tt)          # the context API's step (gather, RK4, scatter)
        ref = group.read()
        J_before = J_d.cpu().numpy().copy()
        if tt < 62:
            E_d.copy_(torch.from_numpy(ref["E"]))
            rc = call_noalloc(stream)
            assert rc == 0, L.omx_last_error(None)
        else:
            side = torch.cuda.Stream(dev)
            side.wait_stream(torch.cuda.current_stream(dev))
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph, stream=side):
                rc = call_noalloc(side.cuda_stream)
            assert rc == 0, L.omx_last_error(None)
            torch.cuda.synchronize()
            assert _rel(rho_d.cpu().numpy(), prev_rho) == 0.0      # capturing ran nothing
            E_d.copy_(torch.from_numpy(ref["E"]))
            graph.replay()
        torch.cuda.synchronize()
        rho, dip = rho_d.cpu().numpy(), dip_d.cpu().numpy()
        prev_rho = rho.copy()
        J, Jo, dJ = J_d.cpu().numpy(), Jo_d.cpu().numpy(), dJ_d.cpu().numpy()
        assert _rel(rho, ref["rho"]) <= TOL and _rel(dip, ref["dipole"]) <= TOL, call
        for c in range(c0, c1 + 1):
            J_ref = wk[:nreal] * ref["dPt_dt"][winner[:nreal], c]
            assert _rel(J[c, :nreal], J_ref) <= TOL, (call, c)
            assert np.array_equal(Jo[c], J_before[c]), (call, c)
            assert _rel(dJ[c, :nreal], (J_ref - J_before[c, :nreal]) / dt) <= TOL, (call, c)
            # points without a writer in this call keep J; their dJ is zero
            assert np.array_equal(J[c, nreal:], J_before[c, nreal:]), (call, c)
            assert np.array_equal(dJ[c, nreal:], np.zeros(2)), (call, c)
        assert np.max(np.abs(J[c0:c1 + 1, :nreal])) > 0.0
        if c0 == 0:       # randomly oriented emitters drive every component
            assert all(np.max(np.abs(J[c, :nreal])) > 0.0 for c in range(3))

    # sizes beyond the fixed scratch array are rejected with a clear error
    rc = L.omx_emitter_step_noalloc(model, MAX_EMITTERS + 1, E_d.data_ptr(), par_d.data_ptr(), rho_d.data_ptr(),
                                     dip_d.data_ptr(), 0, None, None, None, None, None, c0, c1, dt, None)
    assert rc == 1 and b"OMX_NOALLOC_MAX_EMITTERS" in L.omx_last_error(None)
    g.kill()
