"""CPU tests of the differentiable rate network: the FP64 restatement's adjoint
against central finite differences (h = 1e-3) of its own loss, and the C-ABI's
shape validation and workspace sizing (no GPU needed)."""
import numpy as np
import pytest

from oracle import rate_adjoint as ra


def small_case(seed=0, layers=3, rows=6, cols=7, field=5, outputs=3, batch=2, steps=9):
    rng = np.random.default_rng(seed)
    N = rows * cols
    shape = dict(layers=layers, rows=rows, cols=cols, field=field, outputs=outputs,
                 batch=batch, steps=steps, checkpoint=4, dt=1.0)
    x = rng.normal(0, 1, (steps, batch, N))
    w = rng.normal(0, 0.1, (layers - 1, N, field * field))
    R = rng.normal(0, 0.1, (outputs, N))
    tau = rng.uniform(5.0, 15.0, layers)
    target = rng.uniform(0, 1, (batch, outputs))
    return shape, x, w, R, tau, target


@pytest.mark.parametrize("layers", [1, 2, 3])
def test_fp64_adjoint_matches_finite_differences(layers):
    shape, x, w, R, tau, target = small_case(layers=layers)
    loss, dw, dR, dtau, dx = ra.adjoint(shape, x, w, R, tau, target)
    rng = np.random.default_rng(1)
    checks = [("tau", dtau, i) for i in range(layers)]
    checks += [("R", dR, int(i)) for i in rng.choice(dR.size, 6, replace=False)]
    if layers > 1:
        nz = np.flatnonzero(np.abs(dw.reshape(-1)) > 0)
        checks += [("w", dw, int(i)) for i in rng.choice(nz, 8, replace=False)]
    for which, grad, i in checks:
        fd = ra.finite_difference(shape, x, w, R, tau, target, which, i, h=1e-3)
        g = grad.reshape(-1)[i]
        assert abs(g - fd) <= 1e-4 * abs(fd) + 1e-12, (which, i, g, fd)


def test_fp64_input_gradient():
    shape, x, w, R, tau, target = small_case()
    _, _, _, _, dx = ra.adjoint(shape, x, w, R, tau, target)
    h = 1e-3
    for (t, b, i) in [(0, 0, 3), (4, 1, 20), (8, 0, 41)]:
        xp, xm = x.copy(), x.copy()
        xp[t, b, i] += h
        xm[t, b, i] -= h
        fd = (ra.forward(shape, xp, w, R, tau, target)[0] -
              ra.forward(shape, xm, w, R, tau, target)[0]) / (2 * h)
        assert abs(dx[t, b, i] - fd) <= 1e-4 * abs(fd) + 1e-12


def test_rate_shape_validation_and_workspace():
    from synaptogenesis_gb300 import syngen
    net = syngen.RateNetwork(layers=3, rows=64, cols=64, field=5, outputs=10, batch=64,
                             steps=100, checkpoint=10)
    S = 3 * 64 * 4096
    # checkpoints (10) + segment v, r (11 each) + d, lambda (10 each) + carry,
    # plus outputs, readout partials, transposed weights (under 2 S together),
    # plus a segment's per-step weight (10 x 2 x 4096 x 25) and readout
    # (10 x 10 x 4096) gradient totals
    steps = 10 * 2 * 4096 * 25 + 10 * 10 * 4096
    assert net.workspace_bytes >= ((10 + 11 + 11 + 10 + 10 + 1) * S + steps) * 4
    assert net.workspace_bytes < ((10 + 11 + 11 + 10 + 10 + 3) * S + steps) * 4
    for bad in (dict(outputs=17), dict(field=4), dict(field=11), dict(steps=0),
                dict(checkpoint=0), dict(dt=0.0)):
        with pytest.raises(ValueError):
            syngen.RateNetwork(**dict(dict(rows=8, cols=8, batch=2, steps=4), **bad))
