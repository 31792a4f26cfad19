"""Known-answer tests that pin the CPU oracle (no GPU).

The reference ships no tests, golden vectors or fixtures and cannot be compiled here (Fortran
with a hard DFTB+ dependency; no Fortran compiler), so the oracle is pinned by:
  * the reference's literal-precision constants (constants_mod.f90),
  * exact discrete identities of the Yee scheme (single-mode recurrence, PEC energy invariant),
  * physics with closed forms: CPML absorption, Fresnel reflection of Drude and Drude-Lorentz
    media with the reference's ADE susceptibility, Rabi / T1 / T2 dynamics of the emitters,
    linear response of the three-level V system.
"""
import math

import numpy as np
import pytest

from omx.units import UNITS


def test_constants_single_precision_literals(orc):
    c = orc.constants()
    assert c.nm_to_au == float(np.float32(18.897261259077823)) == 18.897260665893555
    assert c.ev_to_au == float(np.float32(1.0) / np.float32(27.2114))
    assert c.alphaCPML == 0.05000000074505806
    assert c.Debye_to_au == float(np.float32(3.0) / np.float32(7.63))
    assert c.eps0 == 1.0 / (4.0 * 3.141592653589793)
    assert abs(1.0 / math.sqrt(c.eps0 * c.mu0) - 137.0) < 1e-12
    # package-side unit table equals the oracle's
    assert UNITS["nm_to_au"] == c.nm_to_au and UNITS["ev_to_au"] == c.ev_to_au


def _au(dr_nm):
    dr = dr_nm * UNITS["nm_to_au"]
    return dr, dr / (2.0 * 137.0)


def test_cpml_tables_shape(orc):
    dr, dt = _au(2.0)
    be, ce, bh, ch, ke, kh = orc.cpml_tables(10, dr, dt)
    assert np.all((be > 0) & (be <= 1)) and np.all((bh > 0) & (bh <= 1))
    assert np.all(ce <= 0) and np.all(ch <= 0)
    assert ke[0] == 5.0 and ke[-1] == 1.0          # kappa grades 5 -> 1 across the layer
    assert np.all(np.diff(ke) < 0) and np.all(np.diff(kh) < 0)


def _mode_recurrence(seq, lam):
    s = np.asarray(seq)
    res = s[2:] + s[:-2] - lam * s[1:-1]
    return np.max(np.abs(res)) / np.max(np.abs(s))


def test_yee_single_mode_recurrence_3d(orc):
    """Ez = sin(kx i) cos(ky j) in a periodic box evolves with e(n+1)+e(n-1) = lam e(n),
    lam = 2 - 4 S^2 (sin^2(kx/2) + sin^2(ky/2)), S = c dt/dr (numerical dispersion)."""
    dr, dt = _au(2.0)
    nx, ny, nz = 16, 8, 4
    g = orc.Grid(3, (nx, ny, nz), 10, (2, 2, 2), dt, dr)
    lo, hi = g.field_bounds(3)
    ez = np.zeros([hi[a] - lo[a] + 1 for a in range(3)])
    kx, ky = 2 * math.pi / nx, 2 * math.pi * 2 / ny
    for i in range(lo[0], hi[0] + 1):
        for j in range(lo[1], hi[1] + 1):
            ez[i - lo[0], j - lo[1], :] = math.sin(kx * i) * math.cos(ky * j)
    g.write_field(3, ez)
    S = 137.0 * dt / dr
    lam = 2.0 - 4.0 * S * S * (math.sin(kx / 2) ** 2 + math.sin(ky / 2) ** 2)
    seq = []
    for tt in range(1, 81):
        g.td_propagate_H_field()
        g.td_propagate_E_field(dt * (tt - 0.5), 0.0)
        seq.append(g.read_field(3)[3 - lo[0], 2 - lo[1], 2 - lo[2]])
    assert _mode_recurrence(seq, lam) < 1e-12


def test_yee_single_mode_recurrence_2d_tmz(orc):
    dr, dt = _au(2.0)
    nx, ny = 12, 10
    g = orc.Grid(2, (nx, ny), 10, (2, 2), dt, dr, mode=1)
    lo, hi = g.field_bounds(3)
    ez = np.zeros([hi[a] - lo[a] + 1 for a in range(3)])
    kx, ky = 2 * math.pi * 1 / nx, 2 * math.pi * 1 / ny
    for i in range(lo[0], hi[0] + 1):
        for j in range(lo[1], hi[1] + 1):
            ez[i - lo[0], j - lo[1], 0] = math.cos(kx * i) * math.sin(ky * j)
    g.write_field(3, ez)
    S = 137.0 * dt / dr
    lam = 2.0 - 4.0 * S * S * (math.sin(kx / 2) ** 2 + math.sin(ky / 2) ** 2)
    seq = []
    for tt in range(1, 81):
        g.td_propagate_H_field()
        g.td_propagate_E_field(dt * (tt - 0.5), 0.0)
        seq.append(g.read_field(3)[4 - lo[0], 3 - lo[1], 0])
    assert _mode_recurrence(seq, lam) < 1e-12


def test_pec_cavity_energy_invariant(orc):
    """Closed (PEC) cavity: W = eps0 |E^n|^2 + mu0 H^{n-1/2}.H^{n+1/2} is conserved by leapfrog."""
    c = orc.constants()
    dr, dt = _au(2.0)
    n = 10
    g = orc.Grid(3, (n, n, n), 10, (1, 1, 1), dt, dr)
    rng = np.random.default_rng(7)
    for f in (1, 2, 3):
        lo, hi = g.field_bounds(f)
        shape = [hi[a] - lo[a] + 1 for a in range(3)]
        e = np.zeros(shape)
        # interior only (ghost planes are the PEC walls)
        e[1 - lo[0]:n + 1 - lo[0], 1 - lo[1]:n + 1 - lo[1], 1 - lo[2]:n + 1 - lo[2]] = rng.standard_normal((n, n, n))
        g.write_field(f, e)
    h_prev = [g.read_field(f) for f in (4, 5, 6)]
    energies = []
    for tt in range(1, 201):
        e_now = [g.read_field(f) for f in (1, 2, 3)]
        g.td_propagate_H_field()
        h_now = [g.read_field(f) for f in (4, 5, 6)]
        W = c.eps0 * sum(float(np.sum(x * x)) for x in e_now) + c.mu0 * sum(
            float(np.sum(a * b)) for a, b in zip(h_prev, h_now))
        energies.append(W)
        g.td_propagate_E_field(dt * (tt - 0.5), 0.0)
        h_prev = h_now
    energies = np.array(energies)
    assert np.max(np.abs(energies - energies[0])) / energies[0] < 1e-11


def _pulse_1d(orc, n, npml, bound, medium=None, m_from=None, w0=None, tau_steps=12, steps=None,
              src_i=None, det_i=None, dr_nm=1.0):
    dr, dt = _au(dr_nm)
    g = orc.Grid(1, (n,), npml, (bound,), dt, dr)
    if medium is not None:
        mm = np.zeros(n, np.int32)
        mm[m_from - 1:n] = 1
        g.set_media([medium], mm)
    src_i = src_i or n // 3
    r0 = (src_i - n // 2 + 0.5) * dr
    tau = tau_steps * dt
    g.add_source("x", 1.0, w0, 4.0 * tau, tau, [r0], 0.0, 0.0, 1e30)
    sig = []
    for tt in range(1, steps + 1):
        time = dt * (tt - 0.5)
        g.td_propagate_H_field()
        g.source_interactions(time)
        g.td_propagate_E_field(time, 0.0)
        sig.append(g.read_field(1)[det_i - 1, 0, 0])
    return np.array(sig), dt


def test_cpml_absorbs_normal_incidence_1d(orc):
    """A pulse running into the 10-cell CPML returns with < 1e-3 of its amplitude; a closed
    (PEC) wall returns all of it."""
    n, npml = 600, 10
    dr, dt = _au(1.0)
    w0 = 2 * math.pi * 137.0 / (20 * dr)   # 20 cells per wavelength
    kw = dict(w0=w0, steps=1400, src_i=400, det_i=200)
    s_cpml, _ = _pulse_1d(orc, n, npml, 3, **kw)
    s_pec, _ = _pulse_1d(orc, n, npml, 1, **kw)
    inc = np.max(np.abs(s_cpml[:700]))
    ref_cpml = np.max(np.abs(s_cpml[900:]))
    ref_pec = np.max(np.abs(s_pec[900:]))
    assert ref_pec > 0.5 * inc
    assert ref_cpml < 1e-3 * inc


def _reflectance(orc, medium_fn, omegas_ev, dr_nm):
    """|r(w)| of a half-space from two 1D runs (vacuum / with medium) at grid spacing dr_nm."""
    scale = int(round(1.0 / dr_nm))
    n, npml = 4000 * scale, 20 * scale
    dr, dt = _au(dr_nm)
    ev = UNITS["ev_to_au"]
    w_c = float(np.mean(omegas_ev)) * ev
    kw = dict(w0=w_c, tau_steps=30 * scale, steps=7000 * scale, src_i=600 * scale, det_i=1000 * scale,
              dr_nm=dr_nm)
    s_vac, _ = _pulse_1d(orc, n, npml, 3, **kw)
    s_med, _ = _pulse_1d(orc, n, npml, 3, medium=medium_fn(dt), m_from=1500 * scale, **kw)
    refl = s_med - s_vac
    t = dt * (np.arange(len(s_vac)) + 1.0)
    out = []
    for wev in omegas_ev:
        ph = np.exp(1j * wev * ev * t)
        out.append(abs(np.sum(refl * ph) / np.sum(s_vac * ph)))
    return np.array(out)


def _fresnel_check(orc, medium_fn, eps_fn, omegas_ev, tol):
    """The staggered grid puts an abrupt interface half a cell off the E node, so |r| converges
    at first order in k*dr: check the two-resolution (Richardson) extrapolation."""
    ev = UNITS["ev_to_au"]
    r1 = _reflectance(orc, medium_fn, omegas_ev, 1.0)
    r2 = _reflectance(orc, medium_fn, omegas_ev, 0.5)
    for q, wev in enumerate(omegas_ev):
        nn = np.sqrt(eps_fn(wev * ev) + 0j)
        r_exact = abs((1 - nn) / (1 + nn))
        e1, e2 = abs(r1[q] - r_exact), abs(r2[q] - r_exact)
        r_extrap = 2.0 * r2[q] - r1[q]
        assert e2 < 0.75 * e1 or e2 < 0.2 * tol * r_exact, (wev, r1[q], r2[q], r_exact)
        assert abs(r_extrap - r_exact) < tol * r_exact, (wev, r_extrap, r_exact)


def test_drude_fresnel_reflection_1d(orc):
    """Drude half-space (wp 9 eV, gamma 1 eV): |r(w)| = |(1-n)/(1+n)|, n^2 = 1 - wp^2/(w^2 + i gamma w).
    The damping keeps the surface-plasma ringing inside the time window of the DFT."""
    ev = UNITS["ev_to_au"]
    wp, gam = 9.0 * ev, 1.0 * ev
    _fresnel_check(orc, lambda dt_: orc.medium_drude(wp, gam, 1.0, dt_),
                   lambda w: 1.0 - wp * wp / (w * w + 1j * gam * w), [11.5, 12.5, 13.5], 0.01)


def test_drude_lorentz_fresnel_reflection_1d(orc):
    """Two-pole Drude-Lorentz medium (eps_inf 5.9, wp 9 eV, poles 2.7/3.9 eV with strengths
    1.0/0.6; damping raised to 1.0/1.0/1.2 eV so the response decays inside the DFT window):
    eps(w) = eps_inf - wp^2/(w^2 + i g w) + sum f_k wp^2/(w_k^2 - w^2 - i g_k w)."""
    ev = UNITS["ev_to_au"]
    wp, g = 9.0 * ev, 1.0 * ev
    poles = [(2.7 * ev, 1.0, 1.0 * ev), (3.9 * ev, 0.6, 1.2 * ev)]

    def eps(w):
        e = 5.9 - wp * wp / (w * w + 1j * g * w)
        for wk, fk, gk in poles:
            e += fk * wp * wp / (wk * wk - w * w - 1j * gk * w)
        return e

    _fresnel_check(orc, lambda dt_: orc.medium_dl_custom(5.9, 9.0, 1.0, [2.7, 3.9], [1.0, 0.6], [1.0, 1.2], dt_),
                   eps, [11.0, 12.0, 13.0], 0.01)


def test_two_level_rabi_t1_t2(orc):
    ev = UNITS["ev_to_au"]
    w0 = 3.0 * ev
    big = 1e30
    # resonant Rabi: p_e(t) = sin^2(mu E0 t / 2); half period flips the population
    mu, E0 = 1.0, 1e-3 * w0
    dt = 0.5
    omega = mu * E0
    nsteps = int(round(math.pi / omega / dt))
    pr = np.array([w0, mu, big, big, 0.0, 0.0, 1.0])
    rho = np.zeros(3)
    for s in range(nsteps):
        rho = orc.emitter_step(1, pr, rho, E0 * math.cos(w0 * (s + 0.5) * dt), dt)
    assert abs(rho[0] - 1.0) < 5e-3
    # Without field the equations are linear, y' = lam y, and classical RK4 advances them by
    # exactly R(lam dt) = 1 + z + z^2/2 + z^3/6 + z^4/24 per step.
    R = lambda z: 1 + z + z * z / 2 + z ** 3 / 6 + z ** 4 / 24
    # T1 decay of the population: lam = -1/T1 (continuum limit exp(-t/T1))
    T1 = 500.0
    pr = np.array([w0, mu, T1, big, 0.0, 0.0, 1.0])
    rho = np.array([0.5, 0.0, 0.0])
    for s in range(400):
        rho = orc.emitter_step(1, pr, rho, 0.0, dt)
    assert abs(rho[0] - 0.5 * R(-dt / T1) ** 400) < 1e-12
    assert abs(rho[0] - 0.5 * math.exp(-400 * dt / T1)) < 1e-9
    # T2 free-induction decay of the coherence: lam = -i w0 - 1/T2
    T2 = 80.0
    pr = np.array([w0, mu, big, T2, 0.0, 0.0, 1.0])
    rho = np.array([0.5, 0.5, 0.0])
    for s in range(400):
        rho = orc.emitter_step(1, pr, rho, 0.0, dt)
    lam = -1j * w0 - 1.0 / T2
    assert abs(complex(rho[1], rho[2]) - 0.5 * R(lam * dt) ** 400) < 1e-12
    assert abs(complex(rho[1], rho[2]) - 0.5 * np.exp(lam * 400 * dt)) < 1e-6


def test_three_level_trace_positivity_and_linear_response(orc):
    ev = UNITS["ev_to_au"]
    deb = UNITS["Debye_to_au"]
    e1, e2, mu1, mu2 = 2.1 * ev, 2.3 * ev, 6.0 * deb, 7.5 * deb
    T1, T2 = 4.0e4, 4.0e3
    dt = 0.14
    rng = np.random.default_rng(3)
    # strong random drive: populations stay in [0,1], rho stays positive semidefinite
    pr3 = np.array([e1, e2, mu1, mu2, T1, T2, 1.0, 0.0, 0.0])
    rho = np.zeros(8)
    for s in range(3000):
        rho = orc.emitter_step(2, pr3, rho, 0.02 * math.sin(0.08 * s) + 0.01 * rng.standard_normal(), dt)
    p1, p2 = rho[0], rho[1]
    p0 = 1 - p1 - p2
    M = np.array([[p0, rho[2] - 1j * rho[3], rho[4] - 1j * rho[5]],
                  [rho[2] + 1j * rho[3], p1, rho[6] - 1j * rho[7]],
                  [rho[4] + 1j * rho[5], rho[6] + 1j * rho[7], p2]])
    assert np.allclose(M, M.conj().T)
    assert np.min(np.linalg.eigvalsh(M)) > -1e-9
    # weak field: the V system responds as the sum of its two transitions
    E_of = lambda s: 1e-6 * math.cos(2.2 * ev * s * dt)
    r3 = np.zeros(8)
    ra = np.zeros(3)
    rb = np.zeros(3)
    pa = np.array([e1, mu1, T1, T2, 1.0, 0.0, 0.0])
    pb = np.array([e2, mu2, T1, T2, 1.0, 0.0, 0.0])
    d3, ds = [], []
    for s in range(4000):
        E = E_of(s)
        r3 = orc.emitter_step(2, pr3, r3, E, dt)
        ra = orc.emitter_step(1, pa, ra, E, dt)
        rb = orc.emitter_step(1, pb, rb, E, dt)
        d3.append(2 * mu1 * r3[2] + 2 * mu2 * r3[4])
        ds.append(2 * mu1 * ra[1] + 2 * mu2 * rb[1])
    d3, ds = np.array(d3), np.array(ds)
    assert np.max(np.abs(d3 - ds)) < 1e-4 * np.max(np.abs(ds))


def test_source_kernel_normalised(orc):
    dr, dt = _au(2.0)
    g = orc.Grid(3, (32, 32, 32), 10, (3, 3, 3), dt, dr)
    s = g.add_source("z", 1.0, 0.1, 10.0, 5.0, [0, 0, 0], 3.0 * dr, 0.0, 1e30)
    import ctypes as C
    ker = np.zeros(7 ** 3)
    nk = C.c_int()
    orc.lib().orc_source_kernel(s, ker.ctypes.data_as(C.POINTER(C.c_double)), C.byref(nk))
    assert nk.value == 3
    assert abs(ker.sum() - 1.0) < 1e-14
    k3 = ker.reshape(7, 7, 7)
    assert np.allclose(k3, k3[::-1, :, :]) and np.allclose(k3, k3.transpose(1, 0, 2))
    assert np.argmax(ker) == (7 ** 3) // 2
