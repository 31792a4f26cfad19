"""Known-answer tests of the frequency-domain oracle (fd_oracle.c, the reference's
apply_operator_3D and BICGStab_L restated), no GPU."""
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
