"""Seeded synthetic input decks with the shapes of the benchmark configurations.

The reference reads its scene from `inp` plus medium/source/detector/q-group side files; a deck
here is the same information as plain arrays (voxel lists in nm, emitter cells and parameters,
detector index lists), produced deterministically from a seed.  `apply_deck` feeds a deck to any
target with the TMxll call surface (the GPU `omx.TMxll`, or the CPU oracle in the tests).

Scene choices where the configuration text leaves a value open are recorded in each builder's
docstring (grid spacing of the 2D and 512^3 scenes, pulse widths, detector fields, T1/T2 of
the three-level molecules, emitter orientation).
"""
import math

import numpy as np

from .units import UNITS, yee_dt

NM = UNITS["nm_to_au"]
EV = UNITS["ev_to_au"]
FS = UNITS["fs_to_au"]
DEBYE = UNITS["Debye_to_au"]

GOLD_DL = dict(kind="dl_custom", eps_inf=5.9, wp=9.0, gamma=0.07, poles=[2.7, 3.9], strengths=[1.0, 0.6],
               widths=[0.3, 0.5])


def _cell_nm(idx, n, dr_nm):
    """Voxel coordinate (nm) that the reference maps onto cell `idx` (int(x/dr) + n/2)."""
    off = np.asarray(idx, dtype=np.float64) - (n // 2)
    return (off + np.where(off >= 0, 0.5, -0.5)) * dr_nm


def _base(dims, n, npml, boundaries, dr_nm, mode=1):
    dr = dr_nm * NM
    return dict(dimensions=dims, grid_Ndims=list(n), npml=npml, boundaries=list(boundaries), mode=mode,
                dr_nm=dr_nm, dr=dr, dt=yee_dt(dr), media=[], voxels=[], sources=[], plane_sources=[],
                groups=[], detectors=[], n_skip=1, t_det_print=1)


def _vacuum_points(rng, n, lo, hi, count, exclude):
    pts = []
    while len(pts) < count:
        p = [int(rng.integers(lo[a], hi[a] + 1)) for a in range(len(n))]
        if not exclude(p):
            pts.append(p)
    return np.array(pts, dtype=np.int32)


def deck_cfg1(n=128, steps=4000, seed=20261204, npml=10, radius_nm=20.0, dr_nm=2.0):
    """Plain 3D FDTD: n^3, dr 2 nm, Courant 0.5, npml 10 CPML on all faces; Drude-Lorentz gold
    sphere (radius 20 nm) at the centre; x-polarised Gaussian-modulated plane-wave soft source at
    2.2 eV, 4 fs FWHM (Ex sheet on the plane k = npml + 4); 16 point Ex detectors at seeded
    random vacuum cells."""
    rng = np.random.default_rng(seed)
    d = _base(3, (n, n, n), npml, (3, 3, 3), dr_nm)
    c = n / 2 + 0.5
    r = radius_nm / dr_nm
    g = np.arange(1, n + 1)
    I, J, K = np.meshgrid(g, g, g, indexing="ij")
    inside = (I - c) ** 2 + (J - c) ** 2 + (K - c) ** 2 <= r * r
    ii, jj, kk = np.nonzero(inside)
    vox = np.stack([_cell_nm(ii + 1, n, dr_nm), _cell_nm(jj + 1, n, dr_nm), _cell_nm(kk + 1, n, dr_nm)], axis=1)
    d["media"].append(dict(GOLD_DL))
    d["voxels"].append(vox)
    tau = 4.0 / (2.0 * math.sqrt(math.log(2.0))) * FS
    d["plane_sources"].append(dict(comp=1, plane_axis=3, plane_index=npml + 4, j_amp=1.0, w0=2.2 * EV,
                                   t0=3.0 * tau, tau=tau, t_init=0.0, t_final=1e30, phase=0.0, chirp=0.0))
    margin = npml + 3
    excl = lambda p: (p[0] - c) ** 2 + (p[1] - c) ** 2 + (p[2] - c) ** 2 <= (r + 2) ** 2 or p[2] <= npml + 6
    pts = _vacuum_points(rng, (n, n, n), [margin] * 3, [n - margin] * 3, 16, excl)
    for p in pts:
        d["detectors"].append(dict(type=1, field=1, idx=p.reshape(1, 3)))
    d["steps"] = steps
    return d


def deck_cfg2(nx=4096, ny=4096, steps=20000, n_emitters=10000, seed=20261205, npml=10, dr_nm=2.0,
              film_nm=40.0, pitch_nm=400.0, hole_nm=150.0, gap_nm=10.0):
    """2D TMz nx x ny, dr 2 nm, periodic in x and CPML in y; 40 nm Drude silver film
    (wp 9.17 eV, gamma 0.021 eV) perforated every 400 nm by 150 nm holes; n_emitters two-level
    emitters (Ez-coupled) at seeded random x, 10 nm above the film, transition energies
    N(3.0, 0.05) eV, dipole 10 D, T1 1 ps, T2 100 fs, one q-group of `material` type with the
    reference's default density factor (1e-3 nm^-3); Gaussian Ez line source at 3.0 eV
    (5 fs envelope) below the film; 16 point Ez detectors at seeded random vacuum cells."""
    rng = np.random.default_rng(seed)
    d = _base(2, (nx, ny), npml, (2, 3, 1), dr_nm, mode=1)
    t_cells = int(round(film_nm / dr_nm))
    j0 = ny // 2 - t_cells // 2
    j1 = j0 + t_cells - 1
    pitch = int(round(pitch_nm / dr_nm))
    hole = int(round(hole_nm / dr_nm))
    i = np.arange(1, nx + 1)
    metal_i = i[((i - 1) % pitch) >= hole]
    jj = np.arange(j0, j1 + 1)
    I, J = np.meshgrid(metal_i, jj, indexing="ij")
    vox = np.stack([_cell_nm(I.ravel(), nx, dr_nm), _cell_nm(J.ravel(), ny, dr_nm)], axis=1)
    d["media"].append(dict(kind="drude", omegaD=9.17, GammaD=0.021, eps_r=1.0))
    d["voxels"].append(vox)
    je = j1 + 1 + int(round(gap_nm / dr_nm))
    ci = rng.integers(1, nx + 1, size=n_emitters).astype(np.int32)
    cells = np.stack([ci, np.full(n_emitters, je, np.int32)], axis=1)
    w0 = rng.normal(3.0, 0.05, size=n_emitters) * EV
    T1 = 1000.0 * FS
    T2 = 100.0 * FS
    params = np.stack([w0, np.full(n_emitters, 10.0 * DEBYE), np.full(n_emitters, T1), np.full(n_emitters, T2),
                       np.zeros(n_emitters), np.zeros(n_emitters), np.ones(n_emitters)], axis=1)
    dt = d["dt"]
    d["groups"].append(dict(group_type=1, model=1, cells=cells, params=params,
                            density=1.0e-3 / NM ** 3, dt=dt * d["n_skip"]))
    tau = 5.0 * FS
    d["plane_sources"].append(dict(comp=3, plane_axis=2, plane_index=npml + 8, j_amp=1.0, w0=3.0 * EV,
                                   t0=3.0 * tau, tau=tau, t_init=0.0, t_final=1e30, phase=0.0, chirp=0.0))
    excl = lambda p: (j0 - 3 <= p[1] <= je + 3)
    pts = _vacuum_points(rng, (nx, ny), [2, npml + 12], [nx - 1, ny - npml - 3], 16, excl)
    for p in pts:
        d["detectors"].append(dict(type=1, field=3, idx=p.reshape(1, 2)))
    d["steps"] = steps
    return d


def deck_cfg3(n=512, steps=30000, n_emitters=100000, seed=20261206, npml=10, dr_nm=1.0):
    """3D n^3 (dr 1 nm), FP32 fields / FP64 emitters: 4x4 array of gold nanorod dimers (rods
    40x10x10 nm along x, 5 nm gaps; Drude-Lorentz gold as in the plain 3D scene), npml 10;
    n_emitters three-level molecules at seeded random cells of the 16 gaps (energies 0,
    N(2.1,0.03), N(2.3,0.03) eV, dipoles U(5,8) D along x, T1 1 ps, T2 100 fs); chirped
    Gaussian Ex sheet 1.8 -> 2.6 eV (10 fs envelope) with a soft-source amplitude that gives
    about 1e8 V/m; 16 point Ex detectors."""
    rng = np.random.default_rng(seed)
    d = _base(3, (n, n, n), npml, (3, 3, 3), dr_nm)
    s = n / 512.0
    rod_l, rod_w, gap = max(4, int(round(40 * s))), max(2, int(round(10 * s))), max(1, int(round(5 * s)))
    pitch_x = max(rod_l * 2 + gap + 4, int(round(110 * s)))
    pitch_y = max(rod_w + 4, int(round(60 * s)))
    x_start = n // 2 - (4 * pitch_x) // 2
    y_start = n // 2 - (4 * pitch_y) // 2
    z0 = n // 2 - rod_w // 2
    vox_cells = []
    gaps = []
    for a in range(4):
        for b in range(4):
            xa = x_start + a * pitch_x + (pitch_x - (2 * rod_l + gap)) // 2
            yb = y_start + b * pitch_y + (pitch_y - rod_w) // 2
            for x0 in (xa, xa + rod_l + gap):
                X, Y, Z = np.meshgrid(np.arange(x0, x0 + rod_l), np.arange(yb, yb + rod_w),
                                      np.arange(z0, z0 + rod_w), indexing="ij")
                vox_cells.append(np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1))
            gaps.append((xa + rod_l, xa + rod_l + gap - 1, yb, yb + rod_w - 1, z0, z0 + rod_w - 1))
    cells3 = np.concatenate(vox_cells)
    vox = np.stack([_cell_nm(cells3[:, q], n, dr_nm) for q in range(3)], axis=1)
    d["media"].append(dict(GOLD_DL))
    d["voxels"].append(vox)
    g = rng.integers(0, len(gaps), size=n_emitters)
    cells = np.zeros((n_emitters, 3), np.int32)
    for q, (x0, x1, y0, y1, zz0, zz1) in enumerate(gaps):
        m = g == q
        cnt = int(m.sum())
        cells[m, 0] = rng.integers(x0, x1 + 1, size=cnt)
        cells[m, 1] = rng.integers(y0, y1 + 1, size=cnt)
        cells[m, 2] = rng.integers(zz0, zz1 + 1, size=cnt)
    e1 = rng.normal(2.1, 0.03, size=n_emitters) * EV
    e2 = rng.normal(2.3, 0.03, size=n_emitters) * EV
    mu1 = rng.uniform(5.0, 8.0, size=n_emitters) * DEBYE
    mu2 = rng.uniform(5.0, 8.0, size=n_emitters) * DEBYE
    T1, T2 = 1000.0 * FS, 100.0 * FS
    params = np.stack([e1, e2, mu1, mu2, np.full(n_emitters, T1), np.full(n_emitters, T2),
                       np.ones(n_emitters), np.zeros(n_emitters), np.zeros(n_emitters)], axis=1)
    d["groups"].append(dict(group_type=1, model=2, cells=cells, params=params, density=1.0e-3 / NM ** 3,
                            dt=d["dt"] * d["n_skip"]))
    tau = 10.0 * FS
    w_lo, w_hi = 1.8 * EV, 2.6 * EV
    chirp = (w_hi - w_lo) / (4.0 * tau)
    c_src = (d["dt"] / UNITS["eps0"]) / d["dr"] / UNITS["c0"] / 2.0
    e_target = 1.0e8 * UNITS["Vm_to_au"]
    d["plane_sources"].append(dict(comp=1, plane_axis=3, plane_index=npml + 4, j_amp=e_target / c_src,
                                   w0=0.5 * (w_lo + w_hi), t0=3.0 * tau, tau=tau, t_init=0.0, t_final=1e30,
                                   phase=0.0, chirp=chirp))
    margin = npml + 3
    excl = lambda p: p[2] <= npml + 6 or abs(p[2] - n / 2) < rod_w + 2
    pts = _vacuum_points(rng, (n, n, n), [margin] * 3, [n - margin] * 3, 16, excl)
    for p in pts:
        d["detectors"].append(dict(type=1, field=1, idx=p.reshape(1, 3)))
    d["steps"] = steps
    return d


def deck_cfg5_instance(n, seed, npml=8, dr_nm=20.0, eps_hi=12.1, fill=0.4):
    """One instance of the batched inverse-design sweep: n^3 grid, npml 8 CPML; seeded binary
    permittivity map (eps 1 / 12.1 at fill 0.4, as a dielectric medium) in the central 50% region;
    a z-directed point dipole source (Blackman-Harris kernel of radius one cell) at the 1.55 um
    vacuum frequency; one point Ez detector."""
    rng = np.random.default_rng(seed)
    d = _base(3, (n, n, n), npml, (3, 3, 3), dr_nm)
    lo, hi = n // 4 + 1, n // 4 + n // 2
    g = np.arange(lo, hi + 1)
    I, J, K = np.meshgrid(g, g, g, indexing="ij")
    on = rng.random(I.shape) < fill
    vox = np.stack([_cell_nm(I[on], n, dr_nm), _cell_nm(J[on], n, dr_nm), _cell_nm(K[on], n, dr_nm)], axis=1)
    d["media"].append(dict(kind="dielectric", eps_r=eps_hi))
    d["voxels"].append(vox)
    w = 1239.84193 / 1550.0 * EV
    tau = 20.0 * FS
    d["sources"].append(dict(dir="z", j_amp=1.0, w0=w, t0=3.0 * tau, tau=tau, r0=[0.0, 0.0, -(n // 3) * dr_nm * NM],
                             radius=1.0 * d["dr"], t_init=0.0, t_final=1e30, phase=0.0, chirp=0.0))
    d["detectors"].append(dict(type=1, field=3, idx=np.array([[n // 2, n // 2, n - npml - 4]], np.int32)))
    return d


def build_medium(spec, dt, factory):
    """Make a medium descriptor with `factory` (the GPU package or the oracle module)."""
    k = spec["kind"]
    if k == "dielectric":
        return factory.medium_dielectric(spec["eps_r"])
    if k == "drude":
        return factory.medium_drude(spec["omegaD"] * EV, spec["GammaD"] * EV, spec["eps_r"], dt)
    if k == "dl_library":
        return factory.medium_dl_library(spec["material"], spec["eps_r"], dt)
    if k == "dl_custom":
        return factory.medium_dl_custom(spec["eps_inf"], spec["wp"], spec["gamma"], spec["poles"],
                                        spec["strengths"], spec["widths"], dt)
    raise ValueError(k)


def media_map(deck, map_fn):
    """map_fn(dims, n, dr, voxel list) -> reference media_map."""
    return map_fn(deck["dimensions"], deck["grid_Ndims"], deck["dr"], deck["voxels"])


def apply_deck(target, deck, factory, mmap, with_groups=True):
    """Register media, sources and q-groups of a deck on a TMxll-like target."""
    media = [build_medium(m, deck["dt"], factory) for m in deck["media"]]
    if media:
        target.set_media(media, mmap)
    for s in deck["sources"]:
        target.add_source(s["dir"], s["j_amp"], s["w0"], s["t0"], s["tau"], s["r0"], s["radius"], s["t_init"],
                          s["t_final"], s["phase"], s["chirp"])
    for p in deck["plane_sources"]:
        target.add_plane_source(p["comp"], p["plane_axis"], p["plane_index"], p["j_amp"], p["w0"], p["t0"],
                                p["tau"], p["t_init"], p["t_final"], p["phase"], p["chirp"])
    groups = []
    if with_groups:
        for g in deck["groups"]:
            groups.append(target.add_q_group(g["group_type"], g["model"], g["cells"], g["params"], g["density"],
                                             g["dt"]))
    return groups
