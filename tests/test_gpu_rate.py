"""GPU tests of the differentiable rate network: forward loss and hand-written
adjoint (weights, readout, time constants, input) against the FP64 CPU
restatement, whose adjoint is itself checked against finite differences;
checkpoint strides change nothing; torch.autograd integration; central finite
differences (h = 1e-3) of the GPU loss; the full 3 x 64x64, batch 64, 100-step
configuration."""
import numpy as np
import pytest

from oracle import rate_adjoint as ra

pytestmark = pytest.mark.gpu

REL = 1e-4     # relative gradient tolerance against FP64


@pytest.fixture(scope="module")
def torch_sg():
    import torch
    from synaptogenesis_gb300 import syngen
    assert torch.cuda.is_available()
    return torch, syngen


def make(seed, layers, rows, cols, field, outputs, batch, steps):
    rng = np.random.default_rng(seed)
    N = rows * cols
    return dict(x=rng.normal(0, 1, (steps, batch, N)).astype(np.float32),
                weights=rng.normal(0, 0.1, (layers - 1, N, field * field)).astype(np.float32),
                readout=rng.normal(0, 0.1, (outputs, N)).astype(np.float32),
                tau=np.full(layers, 10.0, np.float32),
                target=rng.uniform(0, 1, (batch, outputs)).astype(np.float32))


def close(got, want, rel=REL):
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    scale = np.abs(want).max() if want.size else 0.0
    norm = np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-30)
    elem = np.abs(got - want) <= rel * np.abs(want) + rel * scale
    return norm <= rel and bool(elem.all()), norm


def gpu_grads(torch, sg, net, p, steps_dx=True):
    t = {k: torch.tensor(v, device="cuda", requires_grad=k in ("x", "weights", "readout", "tau"))
         for k, v in p.items()}
    loss = net.loss(t["x"], t["weights"], t["readout"], t["tau"], t["target"])
    loss.backward()
    torch.cuda.synchronize()
    return (loss.item(), t["weights"].grad.cpu().numpy(), t["readout"].grad.cpu().numpy(),
            t["tau"].grad.cpu().numpy(), t["x"].grad.cpu().numpy())


@pytest.mark.parametrize("cfg", [
    dict(layers=3, rows=12, cols=10, field=5, outputs=4, batch=3, steps=23, checkpoint=5),
    dict(layers=2, rows=9, cols=9, field=3, outputs=10, batch=5, steps=17, checkpoint=17),
    dict(layers=1, rows=7, cols=11, field=5, outputs=2, batch=2, steps=8, checkpoint=3),
    dict(layers=4, rows=16, cols=16, field=7, outputs=16, batch=2, steps=12, checkpoint=1)])
def test_rate_gradients_match_fp64(torch_sg, cfg):
    torch, sg = torch_sg
    net = sg.RateNetwork(**cfg)
    shape = dict(cfg, dt=1.0)
    p = make(3, cfg["layers"], cfg["rows"], cfg["cols"], cfg["field"], cfg["outputs"],
             cfg["batch"], cfg["steps"])
    loss, dw, dR, dtau, dx = gpu_grads(torch, sg, net, p)
    l64, dw64, dR64, dtau64, dx64 = ra.adjoint(shape, p["x"], p["weights"], p["readout"],
                                               p["tau"], p["target"])
    assert abs(loss - l64) <= 1e-5 * abs(l64)
    for name, g, w in (("weights", dw, dw64), ("readout", dR, dR64), ("tau", dtau, dtau64),
                       ("x", dx, dx64)):
        ok, norm = close(g, w)
        assert ok, (name, norm)


def test_rate_checkpoint_stride_is_exact(torch_sg):
    """Recomputing from checkpoints reproduces the forward states bit for bit."""
    torch, sg = torch_sg
    cfg = dict(layers=3, rows=10, cols=10, field=5, outputs=3, batch=4, steps=20)
    p = make(5, 3, 10, 10, 5, 3, 4, 20)
    results = [gpu_grads(torch, sg, sg.RateNetwork(checkpoint=k, **cfg), p)
               for k in (1, 3, 7, 20, 50)]
    for r in results[1:]:
        for a, b in zip(r, results[0]):
            assert np.array_equal(np.asarray(a), np.asarray(b))


def test_rate_grad_loss_scaling_and_no_input_grad(torch_sg):
    torch, sg = torch_sg
    cfg = dict(layers=2, rows=8, cols=8, field=3, outputs=3, batch=2, steps=10, checkpoint=4)
    net = sg.RateNetwork(**cfg)
    p = make(7, 2, 8, 8, 3, 3, 2, 10)
    _, dw1, dR1, dtau1, _ = gpu_grads(torch, sg, net, p)
    t = {k: torch.tensor(v, device="cuda") for k, v in p.items()}
    for k in ("weights", "readout", "tau"):
        t[k].requires_grad_(True)
    (3.0 * net.loss(t["x"], t["weights"], t["readout"], t["tau"], t["target"])).backward()
    assert t["x"].grad is None
    # grad_loss scales dloss/dy before the adjoint runs, so elements with
    # cancellation round differently from 3 x the unscaled gradient
    for got, want in ((t["weights"].grad, dw1), (t["readout"].grad, dR1), (t["tau"].grad, dtau1)):
        want = 3.0 * want
        np.testing.assert_allclose(got.cpu().numpy(), want, rtol=1e-5,
                                   atol=1e-5 * np.abs(want).max())


def test_rate_finite_differences_on_gpu(torch_sg):
    """Central differences (h = 1e-3) of the float32 GPU loss agree with the
    adjoint.  The loss is float32 (rounding ~3e-8 of ~0.3), so a difference
    quotient with h = 1e-3 carries up to ~1e-4 of absolute noise: that is the
    floor of this check; the strict check is against the FP64 gradient."""
    torch, sg = torch_sg
    cfg = dict(layers=3, rows=12, cols=12, field=5, outputs=4, batch=4, steps=30, checkpoint=10)
    net = sg.RateNetwork(**cfg)
    p = make(11, 3, 12, 12, 5, 4, 4, 30)
    _, dw, dR, dtau, _ = gpu_grads(torch, sg, net, p)
    t = {k: torch.tensor(v, device="cuda") for k, v in p.items()}
    h = 1e-3
    checks = [("tau", l, dtau[l]) for l in range(3)]
    checks += [("readout", i, dR.reshape(-1)[i]) for i in (0, 77, 301, 575)]
    big = np.argsort(-np.abs(dw.reshape(-1)))[:3]
    checks += [("weights", int(i), dw.reshape(-1)[i]) for i in big]
    for name, i, g in checks:
        tp, tm = t[name].clone(), t[name].clone()
        tp.view(-1)[i] += h
        tm.view(-1)[i] -= h
        args = lambda q: [q if k == name else t[k] for k in ("x", "weights", "readout", "tau",
                                                             "target")]
        with torch.no_grad():
            lp = float(net.loss(*args(tp)))
            lm = float(net.loss(*args(tm)))
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g) <= 1e-2 * abs(g) + 1e-4, (name, i, fd, g)


def test_rate_full_configuration_against_fp64(torch_sg):
    """3 x 64x64 layers, convergent 5x5 N(0, 0.1), readout 4096 -> 10, batch 64
    of N(0, 1) sequences, 100 steps, U(0, 1) targets, checkpoint every 10."""
    torch, sg = torch_sg
    cfg = dict(layers=3, rows=64, cols=64, field=5, outputs=10, batch=64, steps=100,
               checkpoint=10)
    net = sg.RateNetwork(**cfg)
    p = make(4, 3, 64, 64, 5, 10, 64, 100)
    loss, dw, dR, dtau, dx = gpu_grads(torch, sg, net, p)
    l64, dw64, dR64, dtau64, dx64 = ra.adjoint(dict(cfg, dt=1.0), p["x"], p["weights"],
                                               p["readout"], p["tau"], p["target"])
    assert abs(loss - l64) <= 1e-5 * abs(l64)
    for name, g, w in (("weights", dw, dw64), ("readout", dR, dR64), ("tau", dtau, dtau64)):
        ok, norm = close(g, w)
        assert ok, (name, norm)
