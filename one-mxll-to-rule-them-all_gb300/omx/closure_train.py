"""Training of the learned emitter closure on trajectories of the plain propagator.

Data: three-level emitters drawn like the 3D nanorod configuration's molecules (levels 0,
N(2.1, 0.03) eV, N(2.3, 0.03) eV; dipoles U(5, 8) D; T1 1 ps, T2 100 fs) under random
band-limited drives E(t) = A * sum_k c_k cos(w_k t + phi_k) / sum_k |c_k|, K frequencies uniform
in [0.5, 4] eV, amplitude A log-uniform in [1e6, 1e9] V/m.  The trajectories come from the GPU
plain propagator (omx_closure_trajectories, the q-groups' own FP64 RK4); the network is trained
on windows of them with the tensor-core training step (omx_closure_train_step).
"""
import numpy as np

from . import Closure, closure_trajectories
from .decks import DEBYE, EV, FS
from .units import UNITS

W = 32                      # window of field samples seen per step


def sample_emitters(n, rng):
    e1 = rng.normal(2.1, 0.03, n) * EV
    e2 = rng.normal(2.3, 0.03, n) * EV
    mu1 = rng.uniform(5.0, 8.0, n) * DEBYE
    mu2 = rng.uniform(5.0, 8.0, n) * DEBYE
    return np.stack([e1, e2, mu1, mu2, np.full(n, 1000.0 * FS), np.full(n, 100.0 * FS), np.ones(n), np.zeros(n),
                     np.zeros(n)], axis=1)


def sample_drives(n, rng, K=8, band_ev=(0.5, 4.0), amp_vm=(1e6, 1e9)):
    amp = np.exp(rng.uniform(np.log(amp_vm[0]), np.log(amp_vm[1]), n)) * UNITS["Vm_to_au"]
    c = rng.uniform(0.2, 1.0, (n, K))
    c /= c.sum(axis=1, keepdims=True)
    w = rng.uniform(band_ev[0], band_ev[1], (n, K)) * EV
    phi = rng.uniform(0.0, 2.0 * np.pi, (n, K))
    drive = np.empty((n, 1 + 3 * K))
    drive[:, 0] = amp
    drive[:, 1::3] = c
    drive[:, 2::3] = w
    drive[:, 3::3] = phi
    return drive


def scales(amp_vm_max=1e9, mu_max_debye=8.0):
    """Field unit: the largest drive amplitude; dipole unit: the largest transition dipole."""
    return amp_vm_max * UNITS["Vm_to_au"], mu_max_debye * DEBYE


def make_data(n, T, dt, seed, K=8):
    """n trajectories of T steps: e [n][T], d [n][T] (scaled) from the plain propagator."""
    rng = np.random.default_rng(seed)
    es, ds = scales()
    return closure_trajectories(2, sample_emitters(n, rng), sample_drives(n, rng, K), T, dt, es, ds)


def batches(e, d, B, T, rng):
    """Random (trajectory, start) windows: inputs e[B][T + W - 1], targets [T][B] (the dipole after
    each of the last T steps)."""
    n, L = e.shape
    while True:
        rows = rng.integers(0, n, B)
        s0 = rng.integers(0, L - (T + W - 1) + 1, B)
        idx = s0[:, None] + np.arange(T + W - 1)[None, :]
        eb = e[rows[:, None], idx]
        db = d[rows[:, None], idx[:, W - 1:]].T
        yield np.ascontiguousarray(eb, np.float32), np.ascontiguousarray(db, np.float32)


def train(closure, e, d, steps, B=1024, T=16, lr=1e-3, skip=4, seed=0, log=None):
    """Adam steps of the tensor-core training step on random windows; returns the losses."""
    rng = np.random.default_rng(seed)
    gen = batches(e, d, B, T, rng)
    losses = []
    for k in range(steps):
        eb, db = next(gen)
        losses.append(closure.train_step(eb, db, lr, skip))
        if log and (k % 50 == 0 or k == steps - 1):
            log(k, losses[-1])
    return losses


def trajectory_batches(e, d, B, rng):
    """Whole trajectories from the ground state: inputs e[B][L], targets [L - W + 1][B] (the dipole
    after each step from the W-th on).  The network's state starts at zero with the emitter's,
    as in a simulation, so back-propagation runs through the whole history it must remember."""
    n = e.shape[0]
    while True:
        rows = rng.integers(0, n, B)
        yield np.ascontiguousarray(e[rows], np.float32), np.ascontiguousarray(d[rows][:, W - 1:].T, np.float32)


def train_trajectories(closure, e, d, steps, B=256, lr=3e-4, skip=4, seed=0, log=None):
    """Adam steps of the tensor-core training step on whole trajectories; returns the losses."""
    rng = np.random.default_rng(seed)
    gen = trajectory_batches(e, d, B, rng)
    losses = []
    for k in range(steps):
        eb, db = next(gen)
        losses.append(closure.train_step(eb, db, lr, skip))
        if log and (k % 100 == 0 or k == steps - 1):
            log(k, losses[-1])
    return losses


def trajectory_errors(predict, e, d, skip=4):
    """Errors of a dipole predictor on whole trajectories e, d [n][L]: predict(e) -> [L - W + 1][n].
    Returns (rms, max): root-mean-square and largest |prediction - target|, both relative to the
    targets' root-mean-square / largest |value| (steps after the first `skip` scored)."""
    t = d[:, W - 1:].T[skip:]
    y = predict(np.ascontiguousarray(e, np.float32))[skip:]
    rms = float(np.sqrt(np.mean((y - t) ** 2)) / max(np.sqrt(np.mean(t ** 2)), 1e-30))
    mx = float(np.max(np.abs(y - t)) / max(np.max(np.abs(t)), 1e-30))
    return rms, mx


def new_closure(seed=0):
    """A closure with the oracle's initialisation rule (uniform +-1/sqrt(fan_in), update gate biased
    to keep its state) and the training data's scales."""
    from math import sqrt

    H, F, G, XH = 128, 256, 512, W + 128
    rng = np.random.default_rng(seed)
    parts = []
    wg = rng.uniform(-1, 1, (G, XH)) / sqrt(XH)
    wg[2 * H:3 * H, W:] = 0.0
    wg[3 * H:, :W] = 0.0
    bg = np.zeros(G)
    bg[H:2 * H] = 1.0
    parts += [wg.ravel(), bg, (rng.uniform(-1, 1, (F, H)) / sqrt(H)).ravel(), np.zeros(F),
              (rng.uniform(-1, 1, (F, F)) / sqrt(F)).ravel(), np.zeros(F),
              (rng.uniform(-1, 1, (F, F)) / sqrt(F)).ravel(), np.zeros(F), rng.uniform(-1, 1, F) / sqrt(F),
              np.zeros(1)]
    es, ds = scales()
    return Closure(np.concatenate(parts).astype(np.float32), es, ds)
