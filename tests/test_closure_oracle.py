"""The FP64 closure oracle's analytic gradient (backward through time) against central finite
differences, on a small batch; no GPU."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import closure_oracle as co  # noqa: E402


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(7)
    B, T, skip = 3, 5, 1
    flat = co.init_params(3) + 0.05 * rng.normal(size=co.n_params()) * np.concatenate(
        [co.wg_mask().ravel(), np.ones(co.n_params() - co.wg_mask().size)])
    e = rng.normal(size=(B, T + co.W - 1))
    target = rng.normal(size=(T, B))
    loss, g = co.loss_and_grad(flat, e, target, T, skip)
    # a spread of coordinates in every parameter block (masked Wg entries have zero gradient)
    offs = np.cumsum([0] + [int(np.prod(s)) for _, s in co.SHAPES])
    idx = []
    for k in range(len(co.SHAPES)):
        idx += list(rng.integers(offs[k], offs[k + 1], 4))
    mask_flat = np.concatenate([co.wg_mask().ravel(), np.ones(co.n_params() - co.wg_mask().size)])
    h = 1e-6
    for i in idx:
        if mask_flat[i] == 0:
            assert g[i] == 0.0
            continue
        fp, fm = flat.copy(), flat.copy()
        fp[i] += h
        fm[i] -= h
        num = (co.loss_and_grad(fp, e, target, T, skip)[0] - co.loss_and_grad(fm, e, target, T, skip)[0]) / (2 * h)
        assert abs(num - g[i]) <= 1e-6 * max(1.0, abs(num)) + 1e-9, (i, num, g[i])
    assert loss > 0
