"""Shared driver for the GPU parity tests: runs one deck through the CUDA library (C-ABI) and
through the CPU oracle with the reference's time-loop ordering (mxim_mxll.f90:92-132)."""
import numpy as np

import omx
from omx import decks


class OracleFactory:
    def __init__(self, orc):
        self.orc = orc

    def medium_dielectric(self, eps_r):
        return self.orc.medium_dielectric(eps_r)

    def medium_drude(self, w, g, e, dt):
        return self.orc.medium_drude(w, g, e, dt)

    def medium_dl_library(self, name, e, dt):
        return self.orc.medium_dl_library(name, e, dt)

    def medium_dl_custom(self, *a):
        return self.orc.medium_dl_custom(*a)


def make_pair(orc, deck, precision="fp64", autotune=False, form=None):
    d = deck
    gpu = omx.TMxll(d["dimensions"], d["grid_Ndims"], d["npml"], d["boundaries"], d["dt"], d["dr"],
                    mode=d["mode"], precision=precision)
    if form is not None:
        gpu.set_step_form(form)
    cpu = orc.Grid(d["dimensions"], d["grid_Ndims"], d["npml"], d["boundaries"], d["dt"], d["dr"], mode=d["mode"])
    mm = decks.media_map(d, omx.media_map_from_voxels) if d["voxels"] else None
    gg = decks.apply_deck(gpu, d, omx, mm)
    cg = decks.apply_deck(cpu, d, OracleFactory(orc), mm)
    for det in d["detectors"]:
        gpu.add_detector(det["type"], det["field"], det["idx"])
    if autotune:
        gpu.autotune(reps=3)
    return gpu, cpu, gg, cg


def step_loop(target, deck, groups, tt0, nsteps, state, sample=None):
    """The reference's loop body for tt = tt0..tt0+nsteps-1; `state` carries tq_step_old/t_skip."""
    dt = deck["dt"]
    n_skip = deck["n_skip"]
    tt_0 = 1 if n_skip == 1 else 0
    for tt in range(tt0, tt0 + nsteps):
        time = dt * (tt - 0.5)
        tq = 1 + (tt - tt_0) // n_skip
        move = False
        if tq > state["tq_old"]:
            state["t_skip"] = time
            state["tq_old"] = tq
            move = len(groups) > 0
        target.td_propagate_H_field()
        target.source_interactions(time)
        target.td_propagate_E_field(time, state["t_skip"])
        if move:
            for g in groups:
                target.q_group_step(g, tq)
        if sample is not None and deck["t_det_print"] and tt % deck["t_det_print"] == 0:
            sample(time)


def oracle_detectors(cpu, deck):
    return np.concatenate([cpu.sample(det["type"], det["field"], det["idx"]) for det in deck["detectors"]])


def run_both(orc, deck, nsteps, precision="fp64", gpu_mode="calls", use_graph=True, autotune=False, form=None):
    gpu, cpu, gg, cg = make_pair(orc, deck, precision, autotune, form)
    st_c = {"tq_old": 0, "t_skip": 0.0}
    trace_c = []
    step_loop(cpu, deck, cg, 1, nsteps, st_c, sample=lambda t: trace_c.append(oracle_detectors(cpu, deck)))
    if gpu_mode == "calls":
        st_g = {"tq_old": 0, "t_skip": 0.0}
        step_loop(gpu, deck, gg, 1, nsteps, st_g, sample=lambda t: gpu.write_detectors_outputs(t))
    else:
        gpu.run(1, nsteps, deck["n_skip"], deck["t_det_print"], use_graph=use_graph)
    times, trace_g = gpu.drain_detectors()
    return gpu, cpu, gg, cg, np.array(trace_c), trace_g


def interior(a, lo, n, dims):
    sl = []
    for ax in range(3):
        if ax < dims:
            sl.append(slice(1 - lo[ax], n[ax] + 1 - lo[ax]))
        else:
            sl.append(slice(None))
    return a[tuple(sl)]


def field_codes(deck):
    if deck["dimensions"] == 3:
        return [1, 2, 3, 4, 5, 6]
    if deck["dimensions"] == 1:
        return [1, 5]
    return [3, 4, 5] if deck["mode"] == 1 else [1, 2, 6]


# Normalisers are floored at FLOOR x the largest one of the comparison: a component or detector
# the wave has not reached yet holds precursor values far below the FP32 range (1e-40 and less),
# which an FP32 run cannot represent; without the floor they would count as full-scale errors.
FLOOR = 1e-6


def compare_fields(gpu, cpu, deck):
    """Max |gpu - oracle| / max|oracle| over the interior of every field component."""
    n = deck["grid_Ndims"]
    pairs = []
    for f in field_codes(deck):
        lo, _ = cpu.field_bounds(f)
        a = interior(gpu.read_field(f), lo, n, deck["dimensions"])
        b = interior(cpu.read_field(f), lo, n, deck["dimensions"])
        pairs.append((np.max(np.abs(a - b)), np.max(np.abs(b))))
    top = max(m for _, m in pairs)
    return float(max(d / max(m, FLOOR * top, 1e-300) for d, m in pairs))


def trace_error(trace_g, trace_c):
    """max relative detector-field error, normalised per detector by the max |field| of its trace."""
    m = np.max(np.abs(trace_c), axis=0)
    scale = np.maximum(m, max(FLOOR * float(np.max(m)), 1e-300))
    return float(np.max(np.abs(trace_g - trace_c) / scale))


def point_trace_error(trace_g, trace_c, deck):
    """Max detector-field error relative to the field at the detector's point: each detector's
    max |gpu - oracle| over the run, divided by the largest |value| that any detector of the same
    point and the same field kind (E: codes 1-3, H: codes 4-6) records.  A component that nearly
    vanishes at its point (for example Hx beside a uniform Ex sheet, 1e-5 of the point's H) holds
    only FP32 rounding of the point's field, which the per-component normalisation of
    trace_error would amplify by that factor in any FP32 implementation."""
    cols = []
    for det in deck["detectors"]:
        kind = 0 if det["field"] <= 3 else 1
        for p in np.asarray(det["idx"]).reshape(-1, np.asarray(det["idx"]).shape[-1]):
            cols.append((tuple(int(v) for v in p), kind))
    assert len(cols) == trace_c.shape[1]
    m = np.max(np.abs(trace_c), axis=0)
    e = np.max(np.abs(trace_g - trace_c), axis=0)
    scale = {}
    for key, v in zip(cols, m):
        scale[key] = max(scale.get(key, 0.0), float(v))
    floor = max(FLOOR * float(np.max(m)), 1e-300)
    return float(max(e[c] / max(scale[key], floor) for c, key in enumerate(cols)))


def tmz_variant_deck(nx, ny, bx, by, with_media=True, src="plane"):
    """2D TMz scene for the FP32 fused step: Drude disc + dielectric block away from CPML,
    a plane or radial Ez source, a material q-group, point detectors."""
    d = decks._base(2, (nx, ny), 6, (bx, by, 1), 2.0, mode=1)
    ev, fs = omx.UNITS["ev_to_au"], omx.UNITS["fs_to_au"]
    if with_media:
        I, J = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), indexing="ij")
        disc = (I - nx * 0.6) ** 2 + (J - ny * 0.5) ** 2 <= (min(nx, ny) * 0.12) ** 2
        block = (np.abs(I - nx * 0.3) < nx * 0.08) & (np.abs(J - ny * 0.55) < ny * 0.1)
        d["media"].append(dict(kind="drude", omegaD=8.5, GammaD=0.2, eps_r=1.5))
        d["voxels"].append(np.stack([decks._cell_nm(I[disc], nx, 2.0), decks._cell_nm(J[disc], ny, 2.0)], axis=1))
        d["media"].append(dict(kind="dielectric", eps_r=3.0))
        d["voxels"].append(np.stack([decks._cell_nm(I[block], nx, 2.0), decks._cell_nm(J[block], ny, 2.0)], axis=1))
    tau = 2.0 * fs
    if src == "plane":
        d["plane_sources"].append(dict(comp=3, plane_axis=2, plane_index=9, j_amp=1.0, w0=2.8 * ev, t0=2.5 * tau,
                                       tau=tau, t_init=0.0, t_final=1e30, phase=0.0, chirp=0.0))
    else:
        d["sources"].append(dict(dir="z", j_amp=1.0, w0=2.8 * ev, t0=2.5 * tau, tau=tau,
                                 r0=[-nx * 0.3 * 2.0 * decks.NM, -ny * 0.3 * 2.0 * decks.NM], radius=2.5 * d["dr"],
                                 t_init=0.0, t_final=1e30, phase=0.1, chirp=0.0))
    rng = np.random.default_rng(nx + ny)
    ne = 30
    cells = np.stack([rng.integers(10, nx - 10, ne), rng.integers(ny // 2 + 12, ny - 10, ne)], axis=1).astype(np.int32)
    par = np.stack([rng.normal(2.8, 0.05, ne) * ev, np.full(ne, 9 * decks.DEBYE), np.full(ne, 400 * fs),
                    np.full(ne, 40 * fs), np.zeros(ne), np.zeros(ne), np.ones(ne)], axis=1)
    d["groups"].append(dict(group_type=1, model=1, cells=cells, params=par, density=3e-3 / decks.NM ** 3, dt=d["dt"]))
    for p in ([3, 5], [nx - 2, ny - 3], [nx // 2, 3 * ny // 4], [1, ny // 2], [nx, 1]):
        for f in (3, 4, 5):
            d["detectors"].append(dict(type=1, field=f, idx=np.array([p], np.int32)))
    return d
