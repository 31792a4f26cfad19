"""Known-answer tests of the frequency-domain oracle (fd_oracle.c, the reference's
apply_operator_1D / 2D / 3D and BICGStab_L restated), no GPU."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import build_oracle  # noqa: E402

build_oracle.build()
import oracle  # noqa: E402

COEF = {1: [-0.5, 0.0, 0.5], 2: [1 / 12, -2 / 3, 0.0, 2 / 3, -1 / 12],
        3: [-1 / 60, 3 / 20, -3 / 4, 0.0, 3 / 4, -3 / 20, 1 / 60],
        4: [1 / 280, -4 / 105, 1 / 5, -4 / 5, 0.0, 4 / 5, -1 / 5, 4 / 105, -1 / 280]}


def interior(A, v):
    g = A.g
    nx, ny, nz = A.n
    return v[:, g:g + nz, g:g + ny, g:g + nx]


@pytest.mark.parametrize("n_der", [1, 2, 3, 4])
def test_plane_wave_matches_the_discrete_derivative(n_der):
    """Periodic box, vacuum: for pl_z = exp(i k y) the operator gives, in pl_x,
    C1 * lambda(k) * pl_z + 0 and in pl_z C2 * pl_z, with lambda(k) = (1/dr) sum_q c_q e^{i k q dr}
    the stencil's exact eigenvalue."""
    n, dr, w0 = (8, 12, 10), 0.5, 0.7
    A = oracle.FDOperator(n, 4, n_der, (2, 2, 2), dr, w0, np.ones((n[0], n[1], n[2]), np.complex128))
    ky = 2 * np.pi * 2 / (n[1] * dr)
    f = A.zeros()
    j = np.arange(1, n[1] + 1)
    wave = np.exp(1j * ky * j * dr)[None, :, None] * np.ones((n[2], 1, n[0]))
    interior(A, f)[2] = wave
    Af = interior(A, A.apply(f))
    q = np.arange(-n_der, n_der + 1)
    lam = np.sum(np.array(COEF[n_der]) / dr * np.exp(1j * ky * q * dr))
    assert np.max(np.abs(Af[0] - 1j * lam * wave)) <= 1e-12 * np.max(np.abs(lam))
    assert np.max(np.abs(Af[2] - (-1j * w0) * wave)) <= 1e-13
    # derivatives of a constant along x and z: the stencil's sum cancels up to rounding
    assert np.max(np.abs(Af[1])) <= 1e-14 and np.max(np.abs(Af[3:])) == 0.0


def test_y_periodic_ghosts_as_in_the_reference():
    """With periodic y the reference copies mi_x only into the low ghost rows and mi_y only into
    the high ones: d(mi_x)/dy at the top row sees zeros above, d(mi_y)/dy at the bottom row too."""
    n, dr, w0 = (4, 6, 4), 1.0, 1.0
    A = oracle.FDOperator(n, 2, 1, (2, 2, 2), dr, w0, np.ones((n[0], n[1], n[2]), np.complex128))
    f = A.zeros()
    interior(A, f)[3] = 1.0          # mi_x constant: its y-derivative vanishes where both sides are copied
    Af = interior(A, A.apply(f))
    # mi_z = +C1 * (dmydx - dmxdy) (with the minus of the mi rows): rows j = 1 .. ny-1 see a constant,
    # row ny sees the zero ghost above: dmxdy = (0 - 1) * 0.5 / dr
    C1 = 1j
    assert np.all(Af[5][:, :-1, :] == 0.0)
    assert np.allclose(Af[5][:, -1, :], -C1 * (0.0 - (-0.5 / dr)), rtol=0, atol=1e-15)


@pytest.mark.parametrize("L", [1, 2, 4])
def test_bicgstab_l_converges_with_pml(L):
    rng = np.random.default_rng(L)
    n, dr, w0 = (10, 9, 8), 0.25, 1.3
    eps = 1.0 + 3.0 * (rng.random((n[0], n[1], n[2])) < 0.3) + 0.05j
    A = oracle.FDOperator(n, 3, 2, (3, 3, 3), dr, w0, eps)
    j = A.zeros()
    interior(A, j)[:] = rng.normal(size=interior(A, j).shape) + 1j * rng.normal(size=interior(A, j).shape)
    f, conv, err, it = A.solve(j, A.zeros(), 1e-10, 1000, L)
    assert conv and err <= 1e-10
    res = interior(A, A.apply(f)) - interior(A, j)
    assert np.linalg.norm(res) <= 1e-9 * np.linalg.norm(interior(A, j))


def interior_nd(A, v):
    g = A.g
    return v[(slice(None),) + tuple(slice(g, g + m) for m in reversed(A.n))]


@pytest.mark.parametrize("n_der", [1, 2, 3])
def test_plane_wave_1d(n_der):
    """1D periodic vacuum: pl_y = exp(i k x) gives -C1 lambda(k) pl_y in pl_x and C2 pl_y in pl_y
    (apply_operator_1D: pl_x = -C1 dpy/dz s + C2 pl_x + ..., pl_y = C1 dpx/dz s + C2 pl_y)."""
    n, dr, w0 = (24,), 0.5, 0.8
    A = oracle.FDOperator(n, 3, n_der, (2,), dr, w0, np.ones(n, np.complex128))
    assert A.shape() == (4, 24 + 2 * n_der)
    k = 2 * np.pi * 3 / (n[0] * dr)
    wave = np.exp(1j * k * np.arange(1, n[0] + 1) * dr)
    f = A.zeros()
    interior_nd(A, f)[1] = wave
    Af = interior_nd(A, A.apply(f))
    q = np.arange(-n_der, n_der + 1)
    lam = np.sum(np.array(COEF[n_der]) / dr * np.exp(1j * k * q * dr))
    assert np.max(np.abs(Af[0] - (-1j) * lam * wave)) <= 1e-12 * np.max(np.abs(lam))
    assert np.max(np.abs(Af[1] - (-1j * w0) * wave)) <= 1e-13
    assert np.max(np.abs(Af[2:])) == 0.0


def test_1d_y_components_carry_no_medium_term():
    """apply_operator_1D adds C3 (eps - C4) Ex to pl_x and mi_x only (as written in the
    reference): constant fields in a periodic dielectric."""
    n, w0 = (10,), 1.1
    eps = np.full(n, 3.0 + 0.5j)
    A = oracle.FDOperator(n, 2, 1, (2,), 0.4, w0, eps)
    f = A.zeros()
    interior_nd(A, f)[0] = 1.0      # pl_x
    interior_nd(A, f)[3] = 1.0      # mi_y
    Af = interior_nd(A, A.apply(f))
    C2, C3 = -1j * w0, -1j * w0 / 2.0
    assert np.allclose(Af[0], C2 + C3 * (eps - 1.0) * 1.0, rtol=0, atol=1e-14)
    assert np.allclose(Af[3], C2, rtol=0, atol=1e-14)                 # no medium term
    assert np.allclose(Af[2], C3 * (eps - 1.0) * 1.0, rtol=0, atol=1e-14)


@pytest.mark.parametrize("n_der", [1, 2])
def test_plane_wave_2d_sign(n_der):
    """2D periodic vacuum: pl_z = exp(i k y) gives -C1 lambda(k) pl_z in pl_x (the 2D operator's
    curl carries the opposite sign of the 3D one, as written in the reference) and C2 pl_z in pl_z."""
    n, dr, w0 = (8, 20), 0.5, 0.7
    A = oracle.FDOperator(n, 3, n_der, (2, 2), dr, w0, np.ones(n, np.complex128))
    assert A.shape() == (6, 20 + 2 * n_der, 8 + 2 * n_der)
    k = 2 * np.pi * 2 / (n[1] * dr)
    wave = np.exp(1j * k * np.arange(1, n[1] + 1) * dr)[:, None] * np.ones((1, n[0]))
    f = A.zeros()
    interior_nd(A, f)[2] = wave
    Af = interior_nd(A, A.apply(f))
    q = np.arange(-n_der, n_der + 1)
    lam = np.sum(np.array(COEF[n_der]) / dr * np.exp(1j * k * q * dr))
    assert np.max(np.abs(Af[0] - (-1j) * lam * wave)) <= 1e-12 * np.max(np.abs(lam))
    assert np.max(np.abs(Af[2] - (-1j * w0) * wave)) <= 1e-13
    assert np.max(np.abs(Af[1])) <= 1e-14 and np.max(np.abs(Af[3:])) == 0.0


@pytest.mark.parametrize("n,bnd", [((60,), (3,)), ((24, 20), (3, 3)), ((20, 18), (2, 3))])
def test_bicgstab_converges_1d_2d(n, bnd):
    rng = np.random.default_rng(len(n))
    eps = 1.0 + 1.25 * (rng.random(n) < 0.3) + 0.05j
    A = oracle.FDOperator(n, 4, 2, bnd, 0.3, 1.2, eps)
    j = A.zeros()
    jv = interior_nd(A, j)
    jv[:] = rng.normal(size=jv.shape) + 1j * rng.normal(size=jv.shape)
    f, conv, err, it = A.solve(j, A.zeros(), 1e-10, 2000, 2)
    assert conv and err <= 1e-10
    res = interior_nd(A, A.apply(f)) - interior_nd(A, j)
    assert np.linalg.norm(res) <= 1e-9 * np.linalg.norm(interior_nd(A, j))
