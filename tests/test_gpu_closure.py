"""Learned emitter closure: the BF16 tensor-core GEMM it is built on (tcgen05 MMA, TMA-staged
operands, FP32 accumulation in tensor memory) against an FP64 numpy product of the same
BF16-rounded inputs.  Products of BF16 values are exact in FP32, so the only error is the FP32
accumulation: the bar is 1e-5 of the largest |D| (K <= 512)."""
import ctypes as C

import numpy as np
import pytest

import omx

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    """float32 -> BF16 bits, round to nearest even."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def bf16_value(b):
    return (b.astype(np.uint32) << 16).view(np.float32)


def act_np(x, act):
    if act == 1:
        return np.tanh(x)
    if act == 2:
        return 1.0 / (1.0 + np.exp(-x))
    if act == 3:
        return np.maximum(x, 0.0)
    return x


@pytest.mark.parametrize("M,N,K,act,bias", [
    (128, 64, 64, 0, False),       # one tile, one K block
    (128, 16, 128, 0, False),      # the narrow N of the closure's output layer
    (300, 384, 256, 1, True),      # GRU gates: ragged M, three column tiles, tanh epilogue
    (1000, 256, 128, 3, True),     # MLP layer, relu
    (77, 130, 96, 2, True),        # ragged everything, K not a multiple of 64
    (4096, 128, 512, 0, False),    # long K (8 blocks through the 4-slot ring)
])
def test_tc_gemm_matches_numpy(M, N, K, act, bias):
    rng = np.random.default_rng(M + N + K)
    a = bf16_bits(rng.normal(size=(M, K)).astype(np.float32))
    b = bf16_bits(rng.normal(size=(N, K)).astype(np.float32))
    bv = rng.normal(size=N).astype(np.float32) if bias else None
    alpha = 0.5
    d = np.zeros((M, N), np.float32)
    lib = omx.lib()
    rc = lib.omx_tc_gemm_bf16(a.ctypes.data_as(C.POINTER(C.c_uint16)), b.ctypes.data_as(C.POINTER(C.c_uint16)),
                              bv.ctypes.data_as(C.POINTER(C.c_float)) if bias else None,
                              d.ctypes.data_as(C.POINTER(C.c_float)), M, N, K, alpha, act)
    assert rc == 0, lib.omx_last_error(None)
    ref = alpha * (bf16_value(a).astype(np.float64) @ bf16_value(b).astype(np.float64).T)
    if bias:
        ref = ref + bv
    ref = act_np(ref, act)
    err = np.max(np.abs(d - ref)) / max(np.max(np.abs(ref)), 1e-30)
    assert err <= 1e-5, err


# ---- the closure network against the FP64 numpy oracle -----------------------------------------
import os  # noqa: E402
import sys  # noqa: E402

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import closure_oracle as co  # noqa: E402


def _scene(B, T, seed):
    rng = np.random.default_rng(seed)
    flat = co.init_params(seed).astype(np.float32)
    # round the weights to BF16 as the device uses them, so that the comparison measures only the
    # BF16 activations and FP32 accumulation
    e = rng.normal(size=(B, T + co.W - 1)).astype(np.float32)
    target = (0.3 * rng.normal(size=(T, B))).astype(np.float32)
    return flat, e, target


def test_closure_parameter_count():
    assert int(omx.lib().omx_closure_n_params()) == co.n_params()


def test_closure_forward_matches_oracle():
    B, T = 64, 6
    flat, e, _ = _scene(B, T, 11)
    cl = omx.Closure(flat)
    y = cl.forward(e, T)
    yref, _ = co.forward(flat.astype(np.float64), e.astype(np.float64), T)
    err = np.max(np.abs(y - yref)) / max(np.max(np.abs(yref)), 1e-30)
    assert err <= 3e-2, err          # BF16 GEMM operands (8 significant bits), FP32 accumulation
    cl.kill()


def test_closure_gradient_matches_oracle():
    """Analytic gradient of the tensor-core backward pass (through time, split-K weight
    gradients) against the FP64 oracle's: per parameter block, cosine >= 0.99 and relative
    norm error <= 8 %.  The oracle's own gradient is pinned by finite differences
    (tests/test_closure_oracle.py)."""
    B, T, skip = 64, 6, 1
    flat, e, target = _scene(B, T, 12)
    cl = omx.Closure(flat)
    loss, g = cl.gradient(e, target, skip)
    lref, gref = co.loss_and_grad(flat.astype(np.float64), e.astype(np.float64), target.astype(np.float64), T, skip)
    assert abs(loss - lref) <= 2e-2 * lref
    offs = np.cumsum([0] + [int(np.prod(s)) for _, s in co.SHAPES])
    for k, (name, _) in enumerate(co.SHAPES):
        a, b = g[offs[k]:offs[k + 1]].astype(np.float64), gref[offs[k]:offs[k + 1]]
        nb = np.linalg.norm(b)
        assert nb > 0, name
        cos = float(a @ b / (np.linalg.norm(a) * nb))
        rel = float(np.linalg.norm(a - b) / nb)
        assert cos >= 0.99 and rel <= 8e-2, (name, cos, rel)
    # masked gate weights get no gradient
    m = co.wg_mask().ravel() == 0
    assert np.all(g[:m.size][m] == 0.0)
    cl.kill()


def test_closure_training_reduces_loss():
    """A learnable target (a causal linear filter of the window plus a cubic term) is fitted:
    60 Adam steps reduce the loss at least 10-fold."""
    B, T = 256, 8
    rng = np.random.default_rng(5)
    e = rng.normal(size=(B, T + co.W - 1)).astype(np.float32)
    k = np.exp(-np.arange(co.W)[::-1] / 6.0) * np.cos(0.7 * np.arange(co.W)[::-1])
    lin = np.stack([e[:, t:t + co.W] @ k for t in range(T)], axis=0) / 4.0
    target = (lin + 0.1 * lin ** 3).astype(np.float32)
    cl = omx.Closure(co.init_params(2).astype(np.float32))
    first = cl.train_step(e, target, 2e-3, skip=0)
    for _ in range(59):
        last = cl.train_step(e, target, 2e-3, skip=0)
    assert last <= first / 10.0, (first, last)
    cl.kill()


# ---- deployment in a q-group: spot check, fallback, graphs --------------------------------------
from omx import decks  # noqa: E402
from gpu_harness import tmz_variant_deck  # noqa: E402

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import oracle as orc_mod  # noqa: E402

E_SCALE, D_SCALE = 1e-4, 1e-3


def _deployed(tol, check_every, frac=0.1, seed=4):
    deck = tmz_variant_deck(128, 96, 2, 3, src="plane")
    g = omx.TMxll(2, deck["grid_Ndims"], deck["npml"], deck["boundaries"], deck["dt"], deck["dr"], mode=omx.TMZ,
                  precision="fp32")
    groups = decks.apply_deck(g, deck, omx, decks.media_map(deck, omx.media_map_from_voxels))
    params = co.init_params(seed).astype(np.float32)
    params[-1] = 0.5               # read-out bias: a visibly wrong network (the plain dipole starts at 0)
    cl = omx.Closure(params, E_SCALE, D_SCALE)
    groups[0].attach_closure(cl, check_fraction=frac, tol=tol, check_every=check_every)
    return deck, g, groups[0], cl


def test_closure_fallback_reseeds_from_the_window():
    """An untrained network fails the first check (after 4 steps); every emitter outside the
    subset restarts from the ground state replayed through its window (here: 28 empty slots and
    the 4 samples seen), the subset keeps its exact plain state, and the plain propagator runs
    from then on.  All compared bit for bit with the oracle's emitter step."""
    deck, g, grp, cl = _deployed(tol=1e-6, check_every=4)
    gd = deck["groups"][0]
    par = np.asarray(gd["params"])
    u = par[:, -3:]
    Eu = []
    for tt in range(1, 7):
        g.run(tt, 1, deck["n_skip"], 0, use_graph=True)
        E = grp.read()["E"]
        Eu.append(u[:, 0] * E[:, 0] + u[:, 1] * E[:, 1] + u[:, 2] * E[:, 2])
        st = grp.closure_status()
        if tt < 4:
            assert not st["fallback"]
        if tt == 4:
            assert st["fallback"] and st["fallback_step"] == 4 and st["checks"] == 1
            rho4 = grp.read()["rho"]
    rho6 = grp.read()["rho"]
    n = par.shape[0]
    for e in range(n):
        r = np.zeros(3)
        window = [0.0] * 28 + [float(np.float32(Eu[s][e] / E_SCALE)) * E_SCALE for s in range(4)]
        if e % 10 == 0:                      # the subset (10 % of 30, spread evenly): exact plain state
            window = [Eu[s][e] for s in range(4)]
        for x in window:
            r = orc_mod.emitter_step(1, par[e], r, x, gd["dt"])
        assert np.array_equal(r, rho4[e]), e
        for s in (4, 5):                     # plain propagator after the fallback
            r = orc_mod.emitter_step(1, par[e], r, Eu[s][e], gd["dt"])
        assert np.array_equal(r, rho6[e]), e
    g.kill()
    cl.kill()


def test_closure_graph_equals_calls_and_check_cadence():
    out = []
    for graph in (True, False):
        deck, g, grp, cl = _deployed(tol=1e30, check_every=5)
        g.run(1, 23, deck["n_skip"], 0, use_graph=graph)
        st = grp.closure_status()
        assert not st["fallback"] and st["checks"] == 4
        r = grp.read()
        out.append((r["dipole"], r["dPt_dt"], g.read_field(3)))
        g.kill()
        cl.kill()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)
    assert np.max(np.abs(out[0][0])) > 0


def test_closure_deployment_matches_forward():
    """The deployed network (window ring, GRU state carried across steps, gates and GRU cell in
    one tensor-core launch) gives the dipoles of omx_closure_forward on the same field history."""
    deck, g, grp, cl = _deployed(tol=1e30, check_every=1000, frac=0.1, seed=6)
    par = np.asarray(deck["groups"][0]["params"])
    u = par[:, -3:]
    n, T = par.shape[0], 12
    eu, dip = [], []
    for tt in range(1, T + 1):
        g.run(tt, 1, deck["n_skip"], 0, use_graph=True)
        r = grp.read()
        eu.append(np.float32((u * r["E"]).sum(1) / E_SCALE))
        dip.append((u * r["dipole"]).sum(1))
    B = (n + 7) // 8 * 8
    e_in = np.zeros((B, T + 31), np.float32)
    e_in[:n, 31:] = np.stack(eu, axis=1)
    y = cl.forward(e_in, T)[:, :n] * D_SCALE
    ref = np.stack(dip, axis=0)
    assert np.max(np.abs(ref)) > 0
    assert np.max(np.abs(y - ref)) <= 1e-5 * np.max(np.abs(ref))
    g.kill()
    cl.kill()


def test_closure_training_gain_on_held_out_trajectories():
    """What training gains: the network trained on whole plain-propagator trajectories (three-level
    emitters under random band-limited drives, as the 3D configuration's molecules) predicts the
    dipoles of fresh trajectories with a fraction of the error of the same network untrained, and
    of the closure-free answer (no induced dipole, error 1 by definition).  At this training
    budget the error stays far above the 1e-3 dipole bar of a deployment, whose spot check then
    hands the group to the plain propagator."""
    from omx import closure_train as ct

    dt = decks.deck_cfg3(n=64, n_emitters=10)["dt"]
    L = 128
    e, d = ct.make_data(4096, L, dt, seed=21)
    eh, dh = ct.make_data(512, L, dt, seed=22)
    T = L - ct.W + 1
    cl = ct.new_closure(seed=1)
    untrained = ct.trajectory_errors(lambda x: cl.forward(x, T), eh, dh)
    ct.train_trajectories(cl, e, d, 600, B=256, lr=3e-4, seed=3)
    trained = ct.trajectory_errors(lambda x: cl.forward(x, T), eh, dh)
    zero = ct.trajectory_errors(lambda x: np.zeros((T, x.shape[0]), np.float32), eh, dh)
    print("closure held-out (rms, max): untrained %s, trained %s, no dipole %s" % (untrained, trained, zero))
    assert zero[0] == pytest.approx(1.0)
    assert trained[0] <= 0.5 * untrained[0], (trained, untrained)
    assert trained[0] <= 0.5 * zero[0], (trained, zero)
    cl.kill()
