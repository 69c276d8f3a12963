"""GPU checks of the smaller neural models beyond their reference fixture
(`models` in tests/golden): the Poisson generator, whose reference draws are
unseeded, against the oracle's restatement of the library's counter-based
draws, and the learning rule the reference cannot run in parallel
structures."""
import numpy as np
import pytest

from tests.golden.cases import Case
from tests.harness import compare, run_library, run_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def syngen():
    from synaptogenesis_gb300 import syngen as sg
    assert sg.get_gpus(), "no CUDA GPU visible"
    return sg


def _poisson_case(steps, rate, seed):
    net = {"structures": [{"name": "g", "type": "parallel", "layers": [
        {"name": "drive", "neural model": "relay", "rows": 32, "columns": 32,
         "init config": {"type": "flat", "value": rate}},
        {"name": "gen", "neural model": "poisson generator", "rows": 32, "columns": 32,
         "seed": seed}]}],
        "connections": [{"name": "d", "from layer": "drive", "to layer": "gen",
                         "type": "one to one", "plastic": False}]}
    return Case("poisson_gen", net, steps, 7, record=[("g", "gen")],
                final=[("neuron", "g", "gen", "output")])


def test_poisson_generator_matches_oracle_and_rate(syngen):
    """Bit-exact spike trains against the oracle's draws over 96 steps (three
    history words), and the spike rate matches the driving probability."""
    case = _poisson_case(96, 0.3, 12345)
    got = run_library(case, syngen)
    want = run_oracle(case)
    assert not compare(got, want)
    raster = (got["rec/g/gen"] >> 31) & 1
    rate = raster[1:].mean()          # the first step reads the zero drive of step -1
    assert abs(rate - 0.3) < 0.01, rate


def test_perceptron_learning_is_refused(syngen):
    """A plastic perceptron connection in a parallel structure: the reference's
    updater reads a source pointer it binds only in feedforward structures;
    here the run is refused with an error, and runs without learning."""
    net = {"structures": [{"name": "s", "layers": [
        {"name": "a", "neural model": "relay", "rows": 2, "columns": 2},
        {"name": "p", "neural model": "perceptron", "rows": 2, "columns": 2}]}],
        "connections": [{"from layer": "a", "to layer": "p", "type": "fully connected"}]}
    n = syngen.Network(net)
    n.build_state()
    report = n.run(syngen.Environment({"modules": []}), {"iterations": 2, "learning flag": True})
    assert report is None or report.obj is None
    assert "perceptron learning" in syngen.last_error()
    report = n.run(syngen.Environment({"modules": []}), {"iterations": 2, "learning flag": False})
    assert report is not None and report.obj is not None, syngen.last_error()


def test_randomized_projection_matches_oracle(syngen):
    """Randomized one-to-one, convergent and divergent projections (seeded
    draws, clipped and wrapping fields, relay and Izhikevich targets):
    bit-exact against the oracle's restatement of the same draws and
    compaction."""
    from tests.test_host_cpu import _randomized_net
    case = Case("randomized", _randomized_net(), 40, 9,
                inputs={"a": lambda rng, t, n: rng.normal(0.0, 5.0, n),
                        "c": lambda rng, t, n: rng.normal(0.0, 5.0, n)},
                record=[("s", "b"), ("s", "iz")],
                final=[("neuron", "s", "b", "input"), ("neuron", "s", "iz", "voltage")])
    got = run_library(case, syngen)
    want = run_oracle(case)
    assert not compare(got, want, nan_keys={"rec/s/b", "neuron/s/b/input", "neuron/s/iz/voltage"})


def test_debug_model_reports_failed_checks(syngen):
    """The debug model's checks (device asserts in the reference) count
    failures on the device; the host reports them as the run's error, and the
    next run, with the dummy value restored, succeeds."""
    from tests.golden.cases import CASES
    case = CASES["debug"]
    net = syngen.Network(case.net)
    net.build_state()
    env = syngen.Environment({"modules": []})
    rep = net.run(env, {"iterations": 3})
    assert rep is not None and rep.obj is not None, syngen.last_error()
    var = net.get_neuron_data("g", "d", "neuron_var").to_np_array()
    assert np.all(var == 1.0)
    var[5] = 2.0
    rep = net.run(env, {"iterations": 2})
    assert rep is None or rep.obj is None
    assert "neuron_var differs" in syngen.last_error() and "index 5" in syngen.last_error()
    var = net.get_neuron_data("g", "d", "neuron_var").to_np_array()
    var[5] = 1.0
    rep = net.run(env, {"iterations": 2})
    assert rep is not None and rep.obj is not None, syngen.last_error()
