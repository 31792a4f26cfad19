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


def make_pair(orc, deck, precision="fp64"):
    d = deck
    gpu = omx.TMxll(d["dimensions"], d["grid_Ndims"], d["npml"], d["boundaries"], d["dt"], d["dr"],
                    mode=d["mode"], precision=precision)
    cpu = orc.Grid(d["dimensions"], d["grid_Ndims"], d["npml"], d["boundaries"], d["dt"], d["dr"], mode=d["mode"])
    mm = decks.media_map(d, omx.media_map_from_voxels) if d["voxels"] else None
    gg = decks.apply_deck(gpu, d, omx, mm)
    cg = decks.apply_deck(cpu, d, OracleFactory(orc), mm)
    for det in d["detectors"]:
        gpu.add_detector(det["type"], det["field"], det["idx"])
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


def run_both(orc, deck, nsteps, precision="fp64", gpu_mode="calls", use_graph=True):
    gpu, cpu, gg, cg = make_pair(orc, deck, precision)
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


def compare_fields(gpu, cpu, deck):
    """Max |gpu - oracle| / max|oracle| over the interior of every field component."""
    worst = 0.0
    n = deck["grid_Ndims"]
    for f in field_codes(deck):
        lo, _ = cpu.field_bounds(f)
        a = interior(gpu.read_field(f), lo, n, deck["dimensions"])
        b = interior(cpu.read_field(f), lo, n, deck["dimensions"])
        scale = max(np.max(np.abs(b)), 1e-300)
        worst = max(worst, float(np.max(np.abs(a - b)) / scale))
    return worst


def trace_error(trace_g, trace_c):
    """max relative detector-field error, normalised per detector by the max |field| of its trace."""
    scale = np.maximum(np.max(np.abs(trace_c), axis=0), 1e-300)
    return float(np.max(np.abs(trace_g - trace_c) / scale))
