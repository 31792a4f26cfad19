#!/usr/bin/env python
"""Benchmark of the time-domain FDTD hot path on GB300.

Workload (default): the 2D TMz configuration -- 4096 x 4096 cells (dr 2 nm), periodic x / CPML y,
a perforated 40 nm Drude silver film, 1e4 two-level emitters (FP64 density matrices) 10 nm above
it, a Gaussian 3.0 eV line source and 16 point detectors sampled every step.  One "step" is one
full time step of the reference's loop (H update, sources, E update with ADE and emitter current,
emitter gather/propagate/scatter, detector sampling).

  value        Gcell-updates/s of the chosen FP32 fused path, device-timed (CUDA events on the
               library's stream) over K steps run by the device-side loop (CUDA graph).
  e2e          the same metric through the reference-facing C-ABI call sequence (per-step calls,
               per-step host->device step scalars and device->host detector samples).
  plain_fp64   the plain FP64 path on the same workload (the speed-up reference) and the FP32
               path's stated error against it (detector fields, emitter dipoles).
  roofline     dominant kernel: algorithmic bytes per launch / mean launch duration (CUDA events).
  cpu_baseline the FP64 CPU oracle (restatement of the reference) on the same workload, a
               bounded sample of steps with all host threads.

--impl reference runs the CPU restatement of the reference on the host cores (the reference
itself is Fortran with an external DFTB+ dependency and no Fortran compiler exists in this image).
--gpus N (torchrun, one process per GPU): independent replicas, weak scaling.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "one-mxll-to-rule-them-all_gb300")
sys.path.insert(0, PKG)

METRIC = "Gcell-updates/s & emitter-steps/s, chosen vs plain form, at stated field error"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2000)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", default="omx", choices=["omx", "reference"])
    p.add_argument("--config", default="cfg2", choices=["cfg1", "cfg2", "cfg3", "cfg4", "cfg5", "fdop"])
    p.add_argument("--instances", type=int, default=64, help="cfg5: number of grids in the batched sweep")
    p.add_argument("--side-min", type=int, default=64, help="cfg5: smallest grid side")
    p.add_argument("--side-max", type=int, default=256, help="cfg5: largest grid side")
    p.add_argument("--train-steps", type=int, default=1500, help="cfg4: Adam steps of the closure training")
    p.add_argument("--trajectories", type=int, default=16384, help="cfg4: training trajectories (plain propagator)")
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-autotune", action="store_true",
                   help="keep the library's default launch shape (a fixed kernel form, e.g. for a profiler)")
    p.add_argument("--grid", type=int, default=None,
                   help="cfg3: cube side instead of 512 (a smaller case of the same scene, e.g. for a profiler)")
    p.add_argument("--skip-plain", action="store_true")
    p.add_argument("--error-steps", type=int, default=None,
                   help="length of the FP32-vs-FP64 error run (default: the configuration's full run)")
    p.add_argument("--no-subrecords", action="store_true",
                   help="cfg2: leave out the records of the 3D configurations (cfg1, cfg3)")
    p.add_argument("--cfg3-error-steps", type=int, default=2000,
                   help="prefix of the 512^3 run over which its FP32 error is stated in the cfg2 line")
    p.add_argument("--sub-cpu-seconds", type=float, default=4.0)
    return p.parse_args()


# ---------------------------------------------------------------------------------- distributed
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x):
        if not self.pg:
            return x
        import torch

        t = torch.tensor([float(x)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples (200 ms) during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------------- workload
def make_deck(cfg, grid=None):
    from omx import decks

    if cfg == "cfg1":
        return decks.deck_cfg1(), "cfg1: 3D 128^3 dr 2 nm, 10-cell CPML, Drude-Lorentz Au sphere r 20 nm, " \
                                  "x-polarised 2.2 eV plane-wave soft source, 16 point detectors"
    if cfg == "cfg4":
        return decks.deck_cfg3(n=384, n_emitters=1_000_000), \
            "cfg4: 3D 384^3 dr 1 nm, 10-cell CPML, 4x4 Au nanorod dimers, 1e6 three-level emitters (plain " \
            "density-matrix propagator), chirped 1.8-2.6 eV drive"
    if cfg == "cfg3":
        n = grid or 512
        ne = 100000 if n == 512 else max(1000, int(100000 * (n / 512) ** 3))
        return decks.deck_cfg3(n=n, n_emitters=ne), \
            f"cfg3: 3D {n}^3 dr 1 nm, 10-cell CPML, 4x4 Au nanorod dimers, {ne} three-level emitters in the gaps, " \
            "chirped 1.8-2.6 eV drive, 16 point detectors"
    return decks.deck_cfg2(), "cfg2: 2D TMz 4096x4096 dr 2 nm, periodic x / CPML y, 40 nm Drude Ag film with " \
                              "150 nm holes at 400 nm pitch, 1e4 two-level emitters, 3.0 eV source, 16 point detectors"


def build_gpu(deck, precision):
    import omx
    from omx import decks

    g = omx.TMxll(deck["dimensions"], deck["grid_Ndims"], deck["npml"], deck["boundaries"], deck["dt"], deck["dr"],
                  mode=deck["mode"], precision=precision)
    mm = decks.media_map(deck, omx.media_map_from_voxels)
    groups = decks.apply_deck(g, deck, omx, mm)
    for det in deck["detectors"]:
        g.add_detector(det["type"], det["field"], det["idx"])
    return g, groups


def cells_of(deck):
    n = 1
    for v in deck["grid_Ndims"]:
        n *= v
    return n


def n_emitters(deck):
    return sum(len(g["cells"]) for g in deck["groups"])


class Loop:
    """The reference's loop state (mxim_mxll.f90:92-104) for the per-call drive."""

    def __init__(self, deck):
        self.deck = deck
        self.tq_old = 0
        self.t_skip = 0.0

    def step(self, target, groups, tt):
        d = self.deck
        time_ = d["dt"] * (tt - 0.5)
        tt_0 = 1 if d["n_skip"] == 1 else 0
        tq = 1 + (tt - tt_0) // d["n_skip"]
        move = False
        if tq > self.tq_old:
            self.t_skip, self.tq_old, move = time_, tq, len(groups) > 0
        target.td_propagate_H_field()
        target.source_interactions(time_)
        target.td_propagate_E_field(time_, self.t_skip)
        if move:
            for g in groups:
                target.q_group_step(g, tq)
        return time_


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def recorded_traffic(key):
    """DRAM bytes per launch of a kernel from the committed ncu summaries (None if absent)."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            e = json.load(f)[key]
        return float(e["dram_bytes_read"] + e["dram_bytes_write"]), e["summary"]
    except (OSError, KeyError, ValueError):
        return None, None


def rel_err(a, b):
    """max over detectors and samples of |a - b| / max|b| of that detector, the normaliser
    floored at 1e-6 of the largest detector's: a detector the pulse has not reached holds
    numerical precursor values (1e-30 and below) that FP32 does not represent."""
    import numpy as np

    m = np.max(np.abs(b), axis=0)
    scale = np.maximum(m, max(1e-6 * float(np.max(m)), 1e-300))
    return float(np.max(np.abs(a - b) / scale))


def error_statement(deck, nsteps, shape=None):
    """The FP32 path (launch shape `shape`, as timed) vs FP64 plain on the same deck over nsteps
    (every detector sampled every step)."""
    import numpy as np

    out = {}
    for prec in ("fp32", "fp64"):
        g, groups = build_gpu(deck, prec)
        if prec == "fp32" and shape is not None:
            g.set_launch_shape(shape)
        g.run(1, nsteps, deck["n_skip"], 1, use_graph=True)
        _, rec = g.drain_detectors(max_records=nsteps)
        dip = groups[0].read()["dipole"] if groups else None
        out[prec] = (rec, dip)
        g.kill()
    field_err = rel_err(out["fp32"][0], out["fp64"][0])
    dip_err = None
    if out["fp64"][1] is not None:
        d32, d64 = out["fp32"][1], out["fp64"][1]
        dip_err = float(np.max(np.abs(d32 - d64)) / max(np.max(np.abs(d64)), 1e-300))
    return field_err, dip_err


# ---------------------------------------------------------------------------------- CPU leg
def cpu_run(deck, seconds, max_steps=None, warmup=1):
    """The FP64 oracle (CPU restatement of the reference) stepping the same workload: `warmup`
    untimed steps, then timed steps until `max_steps` or until `seconds` have passed.  Everything
    on this leg is the oracle's own (media map, media, sources, emitters): the GPU library is not
    loaded."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_oracle

    build_oracle.build()
    import oracle as orc
    from omx import decks       # the seeded deck generator (pure Python, no library)

    g = orc.Grid(deck["dimensions"], deck["grid_Ndims"], deck["npml"], deck["boundaries"], deck["dt"], deck["dr"],
                 mode=deck["mode"])
    mm = decks.media_map(deck, orc.media_map) if deck["voxels"] else None
    groups = decks.apply_deck(g, deck, orc, mm)
    loop = Loop(deck)

    def step(tt):
        loop.step(g, groups, tt)
        for det in deck["detectors"]:
            g.sample(det["type"], det["field"], det["idx"])

    w = max(1, int(warmup))
    for tt in range(1, w + 1):         # warm-up steps outside the clock
        step(tt)
    n, t0 = 0, time.perf_counter()
    while True:
        step(w + 1 + n)
        n += 1
        el = time.perf_counter() - t0
        if (el >= seconds and n >= 2) or (max_steps and n >= max_steps):
            break
    return n, el, orc.lib().orc_num_threads()


def reference_arm_fdop(args):
    """The FP64 C oracle applying the 160^3 frequency-domain operator (same operator and input as
    the GPU arm), a bounded number of applications per timed step."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_oracle

    build_oracle.build()
    import oracle as orc

    rng = np.random.default_rng(CFG5_SEED + 7)
    n, n_der = (160, 160, 160), 2
    eps = 1.0 + 11.1 * (rng.random(n) < 0.4) + 0.0j
    O = orc.FDOperator(n, 8, n_der, (3, 3, 3), 0.05, 2.0 * np.pi / 1.55, eps)
    f = O.zeros()
    g = n_der
    f[:, g:-g, g:-g, g:-g] = 1.0 + 0.5j
    O.apply(f)                          # warm-up application outside the clock
    budget = min(2.0 * args.steps, 150.0)
    k, t0 = 0, time.perf_counter()
    while True:
        O.apply(f)
        k += 1
        el = time.perf_counter() - t0
        if (el >= budget and k >= 2) or k >= args.steps:
            break
    cells = n[0] * n[1] * n[2]
    v = cells * k / el / 1e9
    line = {"impl": "reference", "metric": "frequency-domain operator applications, Gcell/s (and BiCGStab(2) "
            "solve time)", "value": v, "unit": "Gcell-applications/s", "n_gpus": 0, "steps": k, "warmup": 1,
            "ms_per_step": el / k * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128", "data": "synthetic (seeded binary permittivity map)",
            "config": {"workload": "apply_operator_3D on 160^3, n_der 2 (4th order), 8-cell PML, eps 1 / 12.1 "
                                   "(fill 0.4)", "cells": cells},
            "cpu_baseline": {"value": v, "unit": "Gcell-applications/s", "cores": 1, "kind": "port",
                             "sample": f"{k} applications of the C oracle (single-threaded loops)"},
            "e2e": {"value": v, "unit": "Gcell-applications/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def reference_arm(args, dist):
    if dist.rank != 0:
        return
    if args.config == "fdop":
        reference_arm_fdop(args)
        return
    if args.config == "cfg5":
        # the sweep's grids are independent: the sample is its smallest grid
        dks, sides = cfg5_decks(args.instances, args.side_min, args.side_max)
        k = min(range(len(dks)), key=lambda q: sides[q])
        deck, desc = dks[k], "cfg5 sample: the sweep's smallest grid (side %d) of %d" % (sides[k], len(dks))
    else:
        deck, desc = make_deck(args.config, args.grid)
    cells = cells_of(deck)
    # W warm-up steps and K timed steps of the CPU restatement, each bounded: the whole run is
    # sized to finish within a few minutes (about 2 s per timed step at most).
    per_step_budget = 2.0
    W = max(1, args.warmup)
    n, el, cores = cpu_run(deck, seconds=min(per_step_budget * args.steps, 150.0), max_steps=args.steps, warmup=W)
    v = cells * n / el / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "Gcell-updates/s", "n_gpus": 0,
            "steps": n, "warmup": W, "ms_per_step": el / n * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": desc, "cells": cells, "emitters": n_emitters(deck)},
            "cpu_baseline": {"value": v, "unit": "Gcell-updates/s", "cores": cores, "kind": "port",
                             "sample": f"{n} steps of the full workload (FP64 oracle restating the reference)"},
            "e2e": {"value": v, "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------- GPU arm
def measure(args, dist, config, grid, K, W, err_steps, cpu_seconds):
    """One configuration on this GPU: the chosen FP32 path device-timed over K steps of the
    device loop (pre-instantiated CUDA graphs), per-kernel times, the roofline of the dominant
    kernel, the end-to-end C-ABI rates, the plain FP64 path with the FP32 error statement over
    `err_steps` steps, and the CPU oracle on rank 0 (a bounded sample)."""
    import omx

    deck, desc = make_deck(config, grid)
    cells = cells_of(deck)
    ne = n_emitters(deck)
    tdp = deck["t_det_print"]
    dims = deck["dimensions"]

    # ---- chosen path: FP32 (one fused pass per step where eligible), device loop in CUDA
    # graphs; the launch shape from the library's autotuner (timed on the zero initial fields)
    gpu, groups = build_gpu(deck, "fp32")
    shape = gpu.autotune(reps=20) if not args.no_autotune else None
    gpu.run(1, W, deck["n_skip"], tdp, use_graph=True)
    # the step graphs of the timed call are captured and instantiated here, outside the clock
    gpu.prepare_run(1 + W, K, deck["n_skip"], tdp)
    gpu.synchronize()
    dist.barrier()
    clocks = ClockSampler(dist.local_rank)
    clocks.start()
    l0 = gpu.launch_count()
    gpu.timer_start()
    gpu.run(1 + W, K, deck["n_skip"], tdp, use_graph=True)
    ms = gpu.timer_stop()
    launches = gpu.launch_count() - l0
    clk = clocks.stop()
    dist.barrier()
    ms_max = dist.max(ms)
    value = dist.world * cells * K / (ms_max / 1e3) / 1e9
    emitter_rate = dist.world * ne * K / (ms_max / 1e3)
    gpu.drain_detectors()

    # ---- per-kernel durations (events around every launch), same K steps ----------------
    gpu.profile(True)
    gpu.run(1 + W + K, K, deck["n_skip"], tdp, use_graph=False)
    gpu.synchronize()
    per = {}
    for kc, name in ((omx.KC_H, "H"), (omx.KC_E, "E"), (omx.KC_EMIT, "emitters"), (omx.KC_SRC, "sources"),
                     (omx.KC_DET, "detectors")):
        t, n = gpu.profile_query(kc)
        per[name] = {"ms_total": t, "launches": n, "us_per_launch": (t / n * 1e3) if n else None}
    gpu.profile(False)
    gpu.drain_detectors()
    dom = max(("H", "E"), key=lambda k: per[k]["ms_total"])
    kc_dom = omx.KC_H if dom == "H" else omx.KC_E
    kernel_name = {"H": "k_h2/k_h3 (H half-step)", "E": "k_e2/k_e3 (E half-step)"}[dom]
    if per["H"]["launches"] == 0:      # one fused pass per step
        per["fused_HE"] = per.pop("E")
        per.pop("H")
        dom, kernel_name = "fused_HE", ("k_fused3_tma<TY, LEAN_ONLY> + k_f3g_h / k_f3g_e (3D H+E step in one "
                                        "pass split by plane form, lean planes staged by TMA)"
                                        if dims == 3 else
                                        "k_fused_tmz_ws (H+E step in one pass; form from omx_autotune)")
    alg_bytes = gpu.algorithmic_bytes(kc_dom)
    traffic, traffic_src = recorded_traffic("%s %s" % (dom, config + ("" if grid is None else "@%d" % grid)))
    avg_s = per[dom]["ms_total"] / per[dom]["launches"] / 1e3
    peak, peak_kind = peaks()
    achieved = alg_bytes / avg_s / 1e9
    gpu.kill()

    # ---- end to end through the C-ABI: one omx_run call per step (the step's time / source
    # table goes host->device from pinned memory inside the call) and an asynchronous drain of
    # that step's detector samples (device->host into a pinned slot), collected into host arrays
    # two steps later (the drain ring holds four tickets); the last steps' samples are collected
    # before the clock stops ----------------------------------------------------------------------
    npts = sum(len(d["idx"]) for d in deck["detectors"])
    LAG = 2

    def e2e_run(one_step):
        g, grp = build_gpu(deck, "fp32")
        if shape is not None:
            g.set_launch_shape(shape)
        pend = []
        for tt in range(1, W + 1):
            one_step(g, grp, tt, pend)
        while pend:
            g.collect(pend.pop(0))
        g.synchronize()
        dist.barrier()
        t0 = time.perf_counter()
        for tt in range(W + 1, W + K + 1):
            one_step(g, grp, tt, pend)
        while pend:
            g.collect(pend.pop(0))
        g.synchronize()
        el = dist.max(time.perf_counter() - t0)
        g.kill()
        return dist.world * cells * K / el / 1e9

    def drain_step(g, pend):
        pend.append(g.drain_async())
        if len(pend) > LAG:
            g.collect(pend.pop(0))

    def run_step(g, grp, tt, pend):
        g.run(tt, 1, deck["n_skip"], tdp, use_graph=True)
        drain_step(g, pend)

    loop = Loop(deck)

    def call_step(g, grp, tt, pend):
        t_ = loop.step(g, grp, tt)
        g.write_detectors_outputs(t_)
        drain_step(g, pend)

    e2e_value = e2e_run(run_step)
    e2e_calls = e2e_run(call_step)

    # ---- plain FP64 path on the same workload; stated FP32 error against it --------------
    plain = None
    if not args.skip_plain:
        g64, groups64 = build_gpu(deck, "fp64")
        if not args.no_autotune:
            g64.autotune(reps=20)
        g64.run(1, W, deck["n_skip"], tdp, use_graph=True)
        g64.prepare_run(1 + W, K, deck["n_skip"], tdp)
        g64.synchronize()
        g64.timer_start()
        g64.run(1 + W, K, deck["n_skip"], tdp, use_graph=True)
        ms64 = dist.max(g64.timer_stop())
        g64.drain_detectors()
        v64 = dist.world * cells * K / (ms64 / 1e3) / 1e9
        g64.kill()
        field_err, dip_err = error_statement(deck, err_steps, shape)
        plain = {"value": v64, "unit": "Gcell-updates/s", "ms_per_step": ms64 / K,
                 "emitter_steps_per_s": dist.world * ne * K / (ms64 / 1e3),
                 "speedup_fp32_over_fp64": value / v64,
                 "fp32_max_rel_detector_error": field_err, "fp32_max_rel_dipole_error": dip_err,
                 "error_run_steps": err_steps, "configuration_steps": deck["steps"],
                 "error_definition": "max over detectors and steps of |fp32 - fp64| / max|fp64 trace| of that "
                                     "detector (floored at 1e-6 of the largest detector's); dipoles: "
                                     "max |fp32 - fp64| / max |fp64| at the end of the run"}

    # ---- CPU baseline: bounded sample of the oracle on rank 0 --------------------------------
    cpu = None
    if dist.rank == 0 and cpu_seconds > 0:
        n, el, cores = cpu_run(deck, seconds=cpu_seconds)
        cpu = {"value": cells * n / el / 1e9, "unit": "Gcell-updates/s", "cores": cores, "kind": "port",
               "sample": f"{n} full steps of the same workload, FP64 oracle (C restatement of the reference, "
                         f"OpenMP on the bulk loops as in the reference)"}
    if shape is None:
        shape_desc = "library default"
    elif dims == 3 and shape >= 1000:
        shape_desc = "fused 3D pass split by plane form, tile 32 x %d, %d planes per block, ring of %d planes " \
                     "(omx_autotune)" % (shape // 1000 % 100, shape % 1000, shape // 100000 or 4)
    elif dims == 2:
        shape_desc = "fused-kernel form %d (omx_autotune)" % shape
    elif dims == 3:
        shape_desc = "two half-step passes, %d planes marched per thread (omx_autotune: faster than the " \
                     "fused pass at this size)" % shape
    else:
        shape_desc = "planes marched per thread %d (omx_autotune)" % shape
    return {
        "value": value, "ms_per_step": ms_max / K, "steps": K, "warmup": W,
        "config": {"workload": desc, "cells": cells, "emitters": ne, "precision": "fp32 fields, fp64 emitters",
                   "parallelism": f"replicas x{dist.world}" if dist.world > 1 else "single GPU",
                   "l2": "working set %.0f MB > 126 MB L2, no flush" % (cells * (3 if dims == 2 else 6) * 4 / 1e6)
                   if cells * (3 if dims == 2 else 6) * 4 > 126e6 else
                   "working set %.0f MB fits in L2: no flush (the metric is the steady-state rate)" %
                   (cells * 6 * 4 / 1e6),
                   "loop": "device-side loop in pre-instantiated CUDA graphs",
                   "launch_shape": shape_desc},
        "emitter_steps_per_s": emitter_rate,
        "roofline": {"bound": "hbm", "kernel": kernel_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src,
                     "peak_source": peak_kind, "algorithmic_bytes_per_launch": alg_bytes},
        "kernels": per, "plain_fp64": plain, "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "Gcell-updates/s",
                "h2d_bytes_per_step": 8 * (4 + len(deck["sources"]) + len(deck["plane_sources"])),
                "d2h_bytes_per_step": 8 * (npts + 1) + 4,
                "how": "one omx_run call per step (time/source table host->device from pinned memory; the "
                       "step's side-stream work overlaps the next call's first pass) + "
                       "omx_detectors_drain_async of the step's samples and error word (device->host, pinned "
                       "slot) every step, collected into host arrays two steps later",
                "per_call_sequence": {"value": e2e_calls, "unit": "Gcell-updates/s",
                                      "how": "the reference's per-step call sequence through the C-ABI "
                                             "(omx_step_H, omx_source_interactions, omx_step_E, "
                                             "omx_qgroup_step, omx_detectors_record) + asynchronous drain "
                                             "every step; omx_step_H is deferred into the fused pass of "
                                             "omx_step_E"}},
        "gpu_launches": launches, "clocks": clk,
    }


def gpu_arm(args, dist):
    import omx

    if dist.world > 1:
        omx.select_device(dist.local_rank % max(1, omx.device_count()))
    K, W = args.steps, max(3, args.warmup)
    deck, _ = make_deck(args.config, args.grid)
    err_steps = args.error_steps or deck["steps"]
    r = measure(args, dist, args.config, args.grid, K, W, err_steps, args.cpu_seconds)
    others = {}
    if args.config == "cfg2" and not args.no_subrecords:
        # the 3D configurations on the same box, same clock rules: the plain 3D scene at full
        # size and length, the 512^3 dimer scene with its FP32 error over a stated prefix
        others["cfg1"] = measure(args, dist, "cfg1", None, max(K, 200), W, 4000, args.sub_cpu_seconds)
        others["cfg3"] = measure(args, dist, "cfg3", None, K, W, args.cfg3_error_steps, args.sub_cpu_seconds)
    if dist.rank == 0:
        line = {"metric": METRIC, "value": r["value"], "unit": "Gcell-updates/s", "n_gpus": dist.world, "steps": K,
                "warmup": W, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded deck of the configuration's shape)"}
        for k in ("config", "emitter_steps_per_s", "roofline", "kernels", "plain_fp64", "cpu_baseline", "e2e",
                  "gpu_launches", "clocks"):
            line[k] = r[k]
        if others:
            line["other_configs"] = others
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------- cfg5: sweep
CFG5_SEED = 20261208


def cfg5_decks(count, side_min=64, side_max=256):
    """The batched inverse-design sweep: `count` cubic 3D grids whose side is drawn per grid,
    uniformly in [side_min, side_max] (the side, not the volume, is uniform), each with its own
    seeded binary permittivity map, dipole source and Ez detector."""
    import numpy as np

    from omx import decks

    rng = np.random.default_rng(CFG5_SEED)
    sides = [int(x) for x in rng.integers(side_min, side_max + 1, count)]
    return [decks.deck_cfg5_instance(n, seed=CFG5_SEED + 1 + k) for k, n in enumerate(sides)], sides


def batch_shape_text(shape):
    """(the fused batched pass, its tile) from omx_batch_autotune's choice."""
    if shape < 1000:
        return "the two half-step passes of every grid (k_batch3)", "tile depth %d" % shape
    form = shape // 1000 % 1000
    tile = "tile 32 x %d, %d planes per block, ring of %d planes" % (form % 100, shape % 1000, form // 100 or 4)
    s = shape // 1000000
    if s > 0:
        return ("the fused pass of the %d largest grids split by plane form (their general runs' new H, "
                "k_f3g_h_batch, and one k_fused3_batch launch over the other grids' tiles on a second stream "
                "beside one launch of their lean runs, k_fused3_batch_lean, then their general runs' new E, "
                "k_f3g_e_batch)" % s), tile
    return "one k_fused3_batch launch per step over every grid's tiles (largest grid first)", tile


def gpu_arm_cfg5(args, dist):
    import omx

    if dist.world > 1:
        omx.select_device(dist.local_rank % max(1, omx.device_count()))
    line = measure_cfg5(args, dist, args.steps, max(3, args.warmup), args.cpu_seconds)
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def measure_cfg5(args, dist, K, W, cpu_seconds):
    """The batched sweep against the same grids one at a time; the bench line (rank 0) or None."""
    import numpy as np

    import omx

    dks, sides = cfg5_decks(args.instances, args.side_min, args.side_max)
    cells = sum(cells_of(d) for d in dks)
    tdp = 1
    # ---- batched: one persistent launch per pass over all grids, the step in a CUDA graph
    grids = [build_gpu(d, "fp32")[0] for d in dks]
    batch = omx.Batch(grids)
    shape = batch.autotune(reps=3)
    batch.run(1, W, 1, tdp, use_graph=True)
    batch.prepare_run(1 + W, K, 1, tdp)         # tables and step graphs built outside the clock
    batch.synchronize()
    dist.barrier()
    clocks = ClockSampler(dist.local_rank)
    clocks.start()
    l0 = batch.launch_count()
    t0 = time.perf_counter()
    batch.run(1 + W, K, 1, tdp, use_graph=True)
    batch.synchronize()
    t_batch = time.perf_counter() - t0
    launches = batch.launch_count() - l0
    clk = clocks.stop()
    t_batch = dist.max(t_batch)
    traces_b = [g.drain_detectors()[1] for g in grids]
    alg = sum(g.algorithmic_bytes(omx.KC_H) + g.algorithmic_bytes(omx.KC_E) for g in grids)   # per step
    batch.kill()
    for g in grids:
        g.kill()
    # ---- the same grids one at a time (each its own omx_run, CUDA graphs per grid, the graphs
    # captured before the clock) with the batch's arithmetic (traces compared bit for bit), each
    # grid in the fused shape its own autotuner picks (the fused pass only: its bits are the batch's)
    t_solo, same = 0.0, True
    for d, tb in zip(dks, traces_b):
        g = build_gpu(d, "fp32")[0]
        g.set_step_form(omx.STEP_SINGLE_PASS)
        g.autotune(reps=3)
        g.run(1, W, 1, tdp, use_graph=True)
        g.prepare_run(1 + W, K, 1, tdp)
        g.synchronize()
        t0 = time.perf_counter()
        g.run(1 + W, K, 1, tdp, use_graph=True)
        g.synchronize()
        t_solo += time.perf_counter() - t0
        ts = g.drain_detectors()[1]
        same = same and ts.shape == tb.shape and bool(np.array_equal(ts, tb))
        g.kill()
    t_solo = dist.max(t_solo)
    value = dist.world * cells * K / t_batch / 1e9
    solo_value = dist.world * cells * K / t_solo / 1e9
    peak, peak_kind = peaks()
    achieved = alg * K / t_batch / 1e9
    cpu = None
    if dist.rank == 0:
        small = sorted(range(len(dks)), key=lambda k: sides[k])[:2]
        done, el_total, cores, cc = 0, 0.0, 1, 0
        for k in small:
            n, el, cores = cpu_run(dks[k], seconds=cpu_seconds / 2)
            done += n * cells_of(dks[k])
            el_total += el
        cpu = {"value": done / el_total / 1e9, "unit": "Gcell-updates/s", "cores": cores, "kind": "port",
               "sample": "FP64 oracle on the two smallest grids of the sweep (sides %s), %.0f s" %
                         ([sides[k] for k in small], el_total)}
    if dist.rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Gcell-updates/s", "n_gpus": dist.world, "steps": K,
            "warmup": W, "ms_per_step": t_batch / K * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded decks of the configuration's shape)",
            "config": {"workload": "cfg5: %d 3D grids, cubic, side uniform in [%d, %d] per grid (seed %d), "
                                   "8-cell CPML, binary eps 1 / 12.1 map (fill 0.4) in the central 50%%, "
                                   "1.55 um dipole source, one Ez detector each" % (len(dks), args.side_min,
                                                                                    args.side_max, CFG5_SEED),
                       "cells": cells, "sides": sides, "precision": "fp32",
                       "parallelism": f"replicas x{dist.world}" if dist.world > 1 else "single GPU",
                       "l2": "working set %.1f GB > 126 MB L2, no flush" % (cells * 6 * 4 / 1e9),
                       "loop": "omx_batch_run: %s, the steps captured in CUDA graphs; shape from "
                               "omx_batch_autotune: %s" % batch_shape_text(shape),
                       "timing": "wall clock around omx_batch_run + omx_batch_synchronize"},
            "one_at_a_time": {"value": solo_value, "unit": "Gcell-updates/s",
                              "how": "the same grids, each its own omx_run (CUDA graph) in the fused shape "
                                     "its own omx_autotune picks, run one after another",
                              "batch_speedup": value / solo_value,
                              "detector_traces_bit_identical": same,
                              "arithmetic": "one fused pass per grid and step, as the batch"},
            "roofline": {"bound": "hbm", "kernel": batch_shape_text(shape)[0],
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "peak_source": peak_kind,
                         "algorithmic_bytes_per_step": alg,
                         "note": "achieved over the whole step time (sources and detectors included)"},
            "cpu_baseline": cpu,
            "e2e": None,
            "gpu_launches": launches,
            "clocks": clk,
        }
        return line
    return None


# ---------------------------------------------------------------------------------- cfg4: closure
CL_FLOPS_TRAIN = 3 * 2 * (512 * 160 + 256 * 128 + 2 * 256 * 256 + 16 * 256)   # fwd + 2x bwd, per sample-step
CL_FLOPS_INFER = 2 * (512 * 160 + 256 * 128 + 2 * 256 * 256 + 16 * 256)


def gpu_arm_cfg4(args, dist):
    """The learned closure: training throughput of the tensor-core training step on plain-propagator
    trajectories, then the 384^3 grid with 1e6 three-level emitters run with the plain FP64
    propagator and with the trained closure (1 % spot-check subset on the plain propagator)."""
    import numpy as np

    import omx
    from omx import closure_train as ct
    from omx import decks

    if dist.world > 1:
        omx.select_device(dist.local_rank % max(1, omx.device_count()))
    deck = decks.deck_cfg3(n=384, n_emitters=1_000_000)
    dt = deck["dt"] * deck["n_skip"]
    # ---- training data and training throughput
    t0 = time.perf_counter()
    L = 160
    e, d = ct.make_data(args.trajectories, L, dt, seed=CFG5_SEED + 4)
    t_gen = time.perf_counter() - t0
    cl = ct.new_closure(seed=1)
    # whole trajectories from the ground state (back-propagation through all of them), so that
    # the network learns the memory a simulation asks of it
    B, skip = 256, 4
    T = L - ct.W + 1
    eh, dh = ct.make_data(1024, L, dt, seed=CFG5_SEED + 5)
    untrained = ct.trajectory_errors(lambda x: cl.forward(x, T), eh, dh, skip)
    ct.train_trajectories(cl, e, d, 5, B, 3e-4, skip, seed=1)
    t0 = time.perf_counter()
    losses = ct.train_trajectories(cl, e, d, args.train_steps, B, 3e-4, skip, seed=2)
    t_train = time.perf_counter() - t0
    samples = args.train_steps * B * T
    # held-out errors of the trained network on fresh trajectories, against the untrained network
    # and the closure-free answer (no induced dipole)
    trained = ct.trajectory_errors(lambda x: cl.forward(x, T), eh, dh, skip)
    held = trained[1]
    cells = cells_of(deck)
    ne = n_emitters(deck)
    K, W = min(args.steps, 200), max(3, args.warmup)

    def timed(g):
        g.run(1, W, deck["n_skip"], 0, use_graph=True)
        g.prepare_run(1 + W, K, deck["n_skip"], 0)
        g.synchronize()
        dist.barrier()
        g.timer_start()
        g.run(1 + W, K, deck["n_skip"], 0, use_graph=True)
        return dist.max(g.timer_stop())

    # ---- plain FP64 density matrices
    g, groups = build_gpu(deck, "fp32")
    ms_plain = timed(g)
    g.kill()
    # ---- the closure (network on the tensor cores, 1 % spot check, fallback above 1e-3)
    g, groups = build_gpu(deck, "fp32")
    groups[0].attach_closure(cl, check_fraction=0.01, tol=1e-3, check_every=16)
    clocks = ClockSampler(dist.local_rank)
    clocks.start()
    l0 = g.launch_count()
    ms_cl = timed(g)
    launches = g.launch_count() - l0
    clk = clocks.stop()
    status = groups[0].closure_status()
    g.kill()
    # the same with the spot check never falling back, so that the network path is what is timed
    g, groups = build_gpu(deck, "fp32")
    groups[0].attach_closure(cl, check_fraction=0.01, tol=1e30, check_every=16)
    ms_cl_nofb = timed(g)
    status_nofb = groups[0].closure_status()
    g.kill()
    cl.kill()
    if dist.rank == 0:
        value = dist.world * cells * K / (ms_cl_nofb / 1e3) / 1e9
        line = {
            "metric": METRIC, "value": value, "unit": "Gcell-updates/s", "n_gpus": dist.world, "steps": K,
            "warmup": W, "ms_per_step": ms_cl_nofb / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 fields, bf16 network (fp32 accumulation), fp64 spot check",
            "data": "synthetic (seeded deck and seeded drives)",
            "config": {"workload": "cfg4: 3D 384^3 dr 1 nm, 4x4 Au nanorod dimers, 1e6 three-level emitters under "
                                   "the closure (GRU 128 + MLP 3 x 256, window 32), 1 % spot check",
                       "cells": cells, "emitters": ne,
                       "training": {"trajectories": args.trajectories, "steps_per_trajectory": L,
                                    "batch": B, "bptt_steps": T, "adam_steps": args.train_steps,
                                    "scaled_down_from": "2e6 trajectories x 2048 steps"}},
            "emitter_steps_per_s": {"closure": dist.world * ne * K / (ms_cl_nofb / 1e3),
                                    "plain_fp64": dist.world * ne * K / (ms_plain / 1e3)},
            "plain_fp64_propagator": {"value": dist.world * cells * K / (ms_plain / 1e3) / 1e9,
                                      "ms_per_step": ms_plain / K},
            "closure_error": {"spot_check_last": status_nofb["last_error"], "held_out_max": held,
                              "held_out_rms": trained[0], "untrained_rms": untrained[0],
                              "untrained_max": untrained[1], "no_dipole_rms": 1.0,
                              "tolerance": 1e-3, "fallback_at_1e-3": status["fallback"],
                              "fallback_step": status["fallback_step"], "ms_per_step_at_1e-3": ms_cl / K},
            "training": {"samples_per_s": samples / t_train,
                         "tflops": CL_FLOPS_TRAIN * samples / t_train / 1e12,
                         "loss_first": losses[0], "loss_last": losses[-1],
                         "data_generation_s": t_gen,
                         "timing": "wall clock, host batch assembly and transfers included"},
            "roofline": {"bound": "tensor", "kernel": "k_gemm_tc (closure inference GEMMs)",
                         "achieved": CL_FLOPS_INFER * ne * K / (ms_cl_nofb / 1e3) / 1e12, "peak": None,
                         "unit": "TFLOP/s", "frac": None, "traffic": None,
                         "note": "closure flops over the whole step time (field kernels included)"},
            "cpu_baseline": None, "e2e": None, "gpu_launches": launches, "clocks": clk,
        }
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------- fdop
def gpu_arm_fdop(args, dist):
    """The inverse-design program's frequency-domain operator (FP64 complex stencil, order 4 in
    each direction) on a 160^3 grid with 8-cell PML and a binary permittivity map, and a
    BiCGStab(2) solve on a 32^3 grid (permittivity 1 / 2.25 + 0.05i), against the FP64 CPU oracle."""
    import numpy as np

    import omx

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_oracle

    build_oracle.build()
    import oracle as orc

    if dist.world > 1:
        omx.select_device(dist.local_rank % max(1, omx.device_count()))
    rng = np.random.default_rng(CFG5_SEED + 7)
    n, n_der = (160, 160, 160), 2
    eps = 1.0 + 11.1 * (rng.random(n) < 0.4) + 0.0j
    G = omx.FDOperator(n, 8, n_der, (3, 3, 3), 0.05, 2.0 * np.pi / 1.55, eps)
    reps = max(5, min(args.steps, 200))
    ms = dist.max(G.time_apply(reps))
    cells = n[0] * n[1] * n[2]
    # FP64 operations the kernel executes per cell (6 per complex product, 2 per complex add or
    # real scaling): 12 (2n+1)-tap derivative sums (4 per tap), 12 stretch products, the three E
    # sums (6), (eps - C4) C3 (8) and 6 outputs of one difference, three products and two sums (24)
    taps = 2 * n_der + 1
    flops = 12 * taps * 4 + 12 * 6 + 6 + 8 + 6 * 24
    bytes_alg = 16 * (6 + 6 + 1)
    # CPU oracle on the same operator (bounded sample)
    O = orc.FDOperator(n, 8, n_der, (3, 3, 3), 0.05, 2.0 * np.pi / 1.55, eps)
    f = O.zeros()
    g = n_der
    f[:, g:-g, g:-g, g:-g] = 1.0 + 0.5j
    t0 = time.perf_counter()
    k = 0
    while True:
        O.apply(f)
        k += 1
        if time.perf_counter() - t0 >= args.cpu_seconds / 2 or k >= 50:
            break
    cpu_ms = (time.perf_counter() - t0) / k * 1e3
    # a solve on a smaller grid, GPU against the oracle
    ns = (32, 32, 32)
    eps_s = 1.0 + 1.25 * (rng.random(ns) < 0.4) + 0.05j
    Gs = omx.FDOperator(ns, 6, n_der, (3, 3, 3), 0.05, 2.0 * np.pi / 1.55, eps_s)
    Os = orc.FDOperator(ns, 6, n_der, (3, 3, 3), 0.05, 2.0 * np.pi / 1.55, eps_s)
    j = Gs.zeros()
    j[:, g:-g, g:-g, g:-g] = rng.normal(size=j[:, g:-g, g:-g, g:-g].shape)
    t0 = time.perf_counter()
    fg, cg, eg, ig = Gs.solve(j, Gs.zeros(), 1e-8, 2000, 2)
    t_gpu = time.perf_counter() - t0
    t0 = time.perf_counter()
    fo, co, eo, io = Os.solve(j, Os.zeros(), 1e-8, 2000, 2)
    t_cpu = time.perf_counter() - t0
    diff = float(np.linalg.norm(fg - fo) / max(np.linalg.norm(fo), 1e-300))
    G.kill()
    Gs.kill()
    if dist.rank == 0:
        value = dist.world * cells / (ms / 1e3) / 1e9
        line = {
            "metric": "frequency-domain operator applications, Gcell/s (and BiCGStab(2) solve time)",
            "value": value, "unit": "Gcell-applications/s", "n_gpus": dist.world, "steps": reps, "warmup": 2,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic (seeded binary permittivity map)",
            "config": {"workload": "apply_operator_3D on 160^3, n_der 2 (4th order), 8-cell PML, eps 1 / 12.1 "
                                   "(fill 0.4); BiCGStab(2) to 1e-8 on 32^3, eps 1 / 2.25 + 0.05i", "cells": cells},
            "roofline": {"bound": "fp64", "kernel": "k_fd_apply", "achieved": flops * cells / (ms / 1e3) / 1e12,
                         "peak": 1.25, "unit": "TFLOP/s", "frac": flops * cells / (ms / 1e3) / 1e12 / 1.25,
                         "peak_source": "nominal GB300 FP64 (1.25 TFLOP/s dense, FMA counted as 2)",
                         "note": "compiled without FMA contraction for bit parity: one flop per FP64 "
                                 "instruction, so the issue ceiling is half the nominal peak",
                         "frac_of_no_fma_ceiling": flops * cells / (ms / 1e3) / 1e12 / 0.625, "traffic": None,
                         "hbm_gbs_algorithmic": bytes_alg * cells / (ms / 1e3) / 1e9},
            "solve": {"gpu_s": t_gpu, "cpu_oracle_s": t_cpu, "iterations_gpu": ig, "iterations_cpu": io,
                      "converged": [cg, co], "relative_difference": diff},
            "cpu_baseline": {"value": cells / (cpu_ms / 1e3) / 1e9, "unit": "Gcell-applications/s",
                             "cores": 1, "kind": "port",
                             "sample": f"{k} applications of the C oracle (single-threaded loops)"},
            "e2e": None, "gpu_launches": reps + 2,
        }
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    dist = Dist()
    try:
        if args.impl == "reference":
            reference_arm(args, dist)
        elif args.config == "cfg5":
            gpu_arm_cfg5(args, dist)
        elif args.config == "cfg4":
            gpu_arm_cfg4(args, dist)
        elif args.config == "fdop":
            gpu_arm_fdop(args, dist)
        else:
            gpu_arm(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
