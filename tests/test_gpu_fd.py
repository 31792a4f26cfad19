"""The frequency-domain operator (apply_operator_3D) and BiCGStab(L) on the GPU against the FP64
oracle: the operator bit for bit; the solver to its tolerance (its dot products are summed in a
different, deterministic order)."""
import os
import sys

import numpy as np
import pytest

import omx

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import oracle  # noqa: E402

pytestmark = pytest.mark.gpu


def scene(n, n_der, bnd, seed):
    rng = np.random.default_rng(seed)
    eps = 1.0 + 11.1 * (rng.random(n) < 0.4) + 0.02j * rng.random(n)
    return eps, rng


@pytest.mark.parametrize("n,n_der,bnd,transpose", [
    ((17, 12, 9), 1, (2, 2, 2), False),     # all periodic (the y copies of mi_x / mi_y as in the reference)
    ((16, 14, 10), 2, (3, 3, 3), False),    # PML on every face
    ((20, 11, 13), 3, (2, 3, 1), True),     # mixed, adjoint sign
    ((12, 12, 12), 4, (3, 2, 3), False),    # eighth-order stencil, periodic y
])
def test_operator_bit_identical(n, n_der, bnd, transpose):
    eps, rng = scene(n, n_der, bnd, sum(n))
    G = omx.FDOperator(n, 3, n_der, bnd, 0.3, 0.9, eps)
    O = oracle.FDOperator(n, 3, n_der, bnd, 0.3, 0.9, eps)
    f = G.zeros()
    g = n_der
    f[:, g:-g, g:-g, g:-g] = rng.normal(size=f[:, g:-g, g:-g, g:-g].shape) + 1j * rng.normal(
        size=f[:, g:-g, g:-g, g:-g].shape)
    a = G.apply(f, transpose)
    b = O.apply(f, transpose)
    ia, ib = a[:, g:-g, g:-g, g:-g], b[:, g:-g, g:-g, g:-g]
    assert np.max(np.abs(ib)) > 0
    assert np.array_equal(ia, ib)
    G.kill()


@pytest.mark.parametrize("L", [1, 2, 4])
def test_bicgstab_l_matches_oracle(L):
    # a moderate contrast (1 / 2.25) with loss, which BiCGStab(1) also converges on in 1000 steps
    n, n_der, bnd = (12, 10, 9), 2, (3, 3, 3)
    rng = np.random.default_rng(40 + L)
    eps = 1.0 + 1.25 * (rng.random(n) < 0.4) + 0.05j + 0.02j * rng.random(n)
    G = omx.FDOperator(n, 3, n_der, bnd, 0.25, 1.3, eps)
    O = oracle.FDOperator(n, 3, n_der, bnd, 0.25, 1.3, eps)
    j = G.zeros()
    g = n_der
    j[:, g:-g, g:-g, g:-g] = rng.normal(size=j[:, g:-g, g:-g, g:-g].shape) + 1j * rng.normal(
        size=j[:, g:-g, g:-g, g:-g].shape)
    fg, cg, eg, ig = G.solve(j, G.zeros(), 1e-10, 1000, L)
    fo, co, eo, io = O.solve(j, O.zeros(), 1e-10, 1000, L)
    assert co and eo <= 1e-10
    assert cg and eg <= 1e-10, (cg, eg, ig, io)
    res = O.apply(fg)[:, g:-g, g:-g, g:-g] - j[:, g:-g, g:-g, g:-g]
    assert np.linalg.norm(res) <= 1e-9 * np.linalg.norm(j[:, g:-g, g:-g, g:-g])
    d = fg[:, g:-g, g:-g, g:-g] - fo[:, g:-g, g:-g, g:-g]
    assert np.linalg.norm(d) <= 1e-7 * np.linalg.norm(fo[:, g:-g, g:-g, g:-g])
    assert abs(ig - io) <= max(5, io // 5), (ig, io)
    G.kill()


def test_set_eps_replaces_the_permittivity():
    """An optimisation step changes eps_r; the operator after omx_fd_set_eps equals a fresh
    oracle operator on the new map."""
    n, n_der, bnd = (14, 9, 11), 2, (3, 2, 3)
    eps, rng = scene(n, n_der, bnd, 5)
    G = omx.FDOperator(n, 3, n_der, bnd, 0.3, 0.9, eps)
    eps2 = eps + 0.5 * (rng.random(n) < 0.2)
    G.set_eps(eps2)
    O = oracle.FDOperator(n, 3, n_der, bnd, 0.3, 0.9, eps2)
    f = G.zeros()
    g = n_der
    f[:, g:-g, g:-g, g:-g] = rng.normal(size=f[:, g:-g, g:-g, g:-g].shape) + 0.5j
    assert np.array_equal(G.apply(f)[:, g:-g, g:-g, g:-g], O.apply(f)[:, g:-g, g:-g, g:-g])
    G.kill()


def interior_nd(g, v, n):
    return v[(slice(None),) + tuple(slice(g, g + m) for m in reversed(n))]


@pytest.mark.parametrize("n,n_der,bnd,transpose", [
    ((37,), 1, (2,), False),                 # apply_operator_1D, periodic
    ((40,), 3, (3,), True),                  # 1D PML, adjoint sign
    ((21, 17), 2, (2, 2), False),            # apply_operator_2D, periodic on both axes
    ((24, 19), 4, (3, 2), True),             # 2D PML x / periodic y, eighth order, adjoint
    ((18, 26), 1, (3, 3), False),            # 2D PML on every face
])
def test_operator_1d_2d_bit_identical(n, n_der, bnd, transpose):
    rng = np.random.default_rng(sum(n) + n_der)
    eps = 1.0 + 11.1 * (rng.random(n) < 0.4) + 0.02j * rng.random(n)
    G = omx.FDOperator(n, 3, n_der, bnd, 0.3, 0.9, eps)
    O = oracle.FDOperator(n, 3, n_der, bnd, 0.3, 0.9, eps)
    assert G.shape() == O.shape()
    f = G.zeros()
    fi = interior_nd(n_der, f, n)
    fi[:] = rng.normal(size=fi.shape) + 1j * rng.normal(size=fi.shape)
    a = interior_nd(n_der, G.apply(f, transpose), n)
    b = interior_nd(n_der, O.apply(f, transpose), n)
    assert np.max(np.abs(b)) > 0
    assert np.array_equal(a, b)
    G.kill()


@pytest.mark.parametrize("n,bnd", [((80,), (3,)), ((26, 22), (3, 3)), ((20, 24), (2, 3))])
def test_bicgstab_1d_2d_matches_oracle(n, bnd):
    rng = np.random.default_rng(len(n) + 7)
    eps = 1.0 + 1.25 * (rng.random(n) < 0.3) + 0.05j
    G = omx.FDOperator(n, 4, 2, bnd, 0.3, 1.2, eps)
    O = oracle.FDOperator(n, 4, 2, bnd, 0.3, 1.2, eps)
    j = G.zeros()
    ji = interior_nd(2, j, n)
    ji[:] = rng.normal(size=ji.shape) + 1j * rng.normal(size=ji.shape)
    fg, cg, eg, ig = G.solve(j, G.zeros(), 1e-10, 2000, 2)
    fo, co, eo, io = O.solve(j, O.zeros(), 1e-10, 2000, 2)
    assert co and eo <= 1e-10
    assert cg and eg <= 1e-10, (cg, eg, ig, io)
    res = interior_nd(2, O.apply(fg), n) - ji
    assert np.linalg.norm(res) <= 1e-9 * np.linalg.norm(ji)
    d = interior_nd(2, fg - fo, n)
    assert np.linalg.norm(d) <= 1e-7 * np.linalg.norm(interior_nd(2, fo, n))
    G.kill()
