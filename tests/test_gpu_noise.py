"""Init-config noise on the GPU (uniform, normal, Poisson with fixed and
per-neuron random rates, overwriting a layer's input or adding onto an input
layer's): the library's draws equal the oracle's restatement of the same
seeded counter-based generator bit for bit, over several runs of one state
(each layer's step counter lives in the state, so a second run continues the
draws); and at size the draws have their distributions' moments."""
import numpy as np
import pytest

from tests.golden.cases import Case
from tests.harness import run_library, run_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    from synaptogenesis_gb300 import syngen
    assert syngen.get_gpus(), "no CUDA GPU visible"
    syngen.set_warnings(False)
    return syngen


def relay(name, side, init):
    return {"name": name, "neural model": "relay", "rows": side, "columns": side,
            "init config": init}


def noise_case(side=16, steps=12):
    layers = [relay("u", side, {"type": "uniform", "min": -1.0, "max": 2.0, "seed": 3}),
              relay("g", side, {"type": "normal", "mean": 0.5, "std dev": 2.0, "seed": 4}),
              relay("p", side, {"type": "poisson", "rate": 200, "value": 3.0, "seed": 5}),
              relay("q", side, {"type": "poisson", "rate": 400, "value": 1.0, "random": True}),
              relay("inp", side, {"type": "poisson", "rate": 300, "value": 2.5, "seed": 6})]
    net = {"structures": [{"name": "n", "type": "parallel", "layers": layers}],
           "connections": []}
    names = [l["name"] for l in layers]
    return Case("noise", net, steps, 17, inputs={"inp": lambda rng, t, m: rng.normal(0, 1, m)},
                record=[("n", l) for l in names],
                final=[("neuron", "n", l, "input") for l in names], learning=False)


def test_noise_matches_oracle(sg):
    case = noise_case()
    got = run_library(case, sg)
    want = run_oracle(case)
    for k, w in want.items():
        assert np.array_equal(got[k], w), k
    assert np.any(want["rec/n/p"] != 0) and np.any(want["rec/n/q"] != 0)


def test_noise_continues_across_runs(sg):
    """Two runs of 6 steps draw what one run of 12 does."""
    case = noise_case(steps=12)
    want = run_oracle(case)
    net_dict = case.net
    net = sg.Network(net_dict)
    net.build_state()
    rng = np.random.default_rng(case.seed + 1000)
    frames = {l: [] for _, l in case.record}
    names = [l for _, l in case.record]

    def in_cb(ID, size, ptr):
        sg.FloatArray(size, ptr).to_np_array()[:] = rng.normal(0, 1, size).astype(np.float32)

    def out_cb(ID, size, ptr):
        frames[names[ID]].append(sg.FloatArray(size, ptr).to_np_array().view(np.uint32).copy())

    sg.create_io_callback("noise_in", in_cb)
    sg.create_io_callback("noise_out", out_cb)
    env = sg.Environment({"modules": [
        {"type": "callback", "layers": [{"structure": "n", "layer": "inp", "input": True,
                                         "function": "noise_in", "id": 0}]},
        {"type": "callback", "layers": [{"structure": "n", "layer": l, "output": True,
                                         "function": "noise_out", "id": i}
                                        for i, l in enumerate(names)]}]})
    for _ in range(2):
        rep = net.run(env, {"iterations": 6, "learning flag": False})
        assert rep is not None and rep.obj is not None
    for l in names:
        assert np.array_equal(np.stack(frames[l]), want["rec/n/" + l]), l


def test_noise_moments_at_size(sg):
    side = 256
    layers = [relay("g", side, {"type": "normal", "mean": -1.0, "std dev": 3.0, "seed": 8}),
              relay("u", side, {"type": "uniform", "min": 0.0, "max": 4.0, "seed": 9}),
              relay("q", side, {"type": "poisson", "rate": 100, "value": 1.0, "random": True,
                                "seed": 10})]
    net = sg.Network({"structures": [{"name": "n", "type": "parallel", "layers": layers}],
                      "connections": []})
    net.build_state()
    fires = []
    env = sg.Environment({"modules": []})
    for _ in range(4):
        net.run(env, {"iterations": 1, "learning flag": False})
        g = net.get_neuron_data("n", "g", "input").to_np_array().astype(np.float64)
        u = net.get_neuron_data("n", "u", "input").to_np_array().astype(np.float64)
        q = net.get_neuron_data("n", "q", "input").to_np_array()
        assert abs(g.mean() + 1.0) < 0.05 and abs(g.std() - 3.0) < 0.05
        assert abs(u.mean() - 2.0) < 0.02 and abs(u.var() - 16.0 / 12.0) < 0.03
        fires.append(q.mean())
    # per-neuron rates uniform in [0, 0.1): mean firing probability 0.05
    assert abs(np.mean(fires) - 0.05) < 0.003
