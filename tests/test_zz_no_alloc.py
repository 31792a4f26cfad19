"""The emitter step that allocates nothing (omx_emitter_step_noalloc), for callers that cannot
call cudaMalloc: it must give what the context API's q-group step gives for the same inputs.

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


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _scene():
    deck = decks.deck_cfg2(nx=128, ny=96, n_emitters=80, npml=8, pitch_nm=100.0, hole_nm=30.0, film_nm=20.0)
    g = omx.TMxll(2, deck["grid_Ndims"], deck["npml"], deck["boundaries"], deck["dt"], deck["dr"], mode=omx.TMZ,
                  precision="fp64")
    groups = decks.apply_deck(g, deck, omx, decks.media_map(deck, omx.media_map_from_voxels))
    return deck, g, groups[0]


def _advance(g, deck, group, state, tt, with_q=True):
    time = deck["dt"] * (tt - 0.5)
    state["t_skip"] = time                     # n_skip = 1: every step is a quantum step
    g.td_propagate_H_field()
    g.source_interactions(time)
    g.td_propagate_E_field(time, state["t_skip"])
    if with_q:
        g.q_group_step(group, tt)


def test_noalloc_emitter_step_matches_qgroup_step():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    L = omx.lib()
    deck, g, group = _scene()
    gd = deck["groups"][0]
    n = len(gd["cells"])
    # current points of a `material` group: the distinct emitter cells; the last emitter in a
    # cell writes it (interactions_mod.f90:1181-1190)
    keys = [tuple(c) for c in gd["cells"]]
    uniq = sorted(set(keys))
    slot = {k: p for p, k in enumerate(uniq)}
    winner = np.full(len(uniq), -1, np.int32)
    for e, k in enumerate(keys):
        winner[slot[k]] = e
    wk = np.full(len(uniq), gd["density"])
    npnt = len(uniq)
    dt = gd["dt"]

    state = {"t_skip": 0.0}
    for tt in range(1, 60):
        _advance(g, deck, group, state, tt)
    prev = group.read()
    J_prev = np.zeros((3, npnt))
    J_prev[2] = wk * prev["dPt_dt"][winner, 2]

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

    for call, tt in enumerate((60, 61)):
        _advance(g, deck, group, state, tt)          # the context API's step (gather, RK4, scatter)
        ref = group.read()
        E_d.copy_(torch.from_numpy(ref["E"]))
        J_before = J_d.cpu().numpy().copy()
        rc = L.omx_emitter_step_noalloc(omx.TWO_LEVEL, n, E_d.data_ptr(), par_d.data_ptr(), rho_d.data_ptr(),
                                         dip_d.data_ptr(), npnt, win_d.data_ptr(), wk_d.data_ptr(), J_d.data_ptr(),
                                         Jo_d.data_ptr(), dJ_d.data_ptr(), 2, 2, dt, C.c_void_p(stream))
        assert rc == 0, L.omx_last_error(None)
        torch.cuda.synchronize()
        rho, dip = rho_d.cpu().numpy(), dip_d.cpu().numpy()
        J, Jo, dJ = J_d.cpu().numpy(), Jo_d.cpu().numpy(), dJ_d.cpu().numpy()
        assert _rel(rho, ref["rho"]) <= TOL and _rel(dip, ref["dipole"]) <= TOL, call
        J_ref = wk * ref["dPt_dt"][winner, 2]
        assert _rel(J[2], J_ref) <= TOL, call
        assert np.array_equal(Jo[2], J_before[2]), call
        assert _rel(dJ[2], (J_ref - J_before[2]) / dt) <= TOL, call
        assert np.max(np.abs(J_ref)) > 0.0

    # sizes beyond the fixed scratch array are rejected with a clear error
    big = 65536 + 1
    rc = L.omx_emitter_step_noalloc(omx.TWO_LEVEL, big, E_d.data_ptr(), par_d.data_ptr(), rho_d.data_ptr(),
                                     dip_d.data_ptr(), 0, None, None, None, None, None, 2, 2, dt, None)
    assert rc == 1 and b"OMX_NOALLOC_MAX_EMITTERS" in L.omx_last_error(None)
    g.kill()
