"""GPU parity: every golden case through the C-ABI against the reference's own
recorded results (bit-exact), and against the oracle.

Bit-exact: spike rasters, output-history words, voltages, recoveries,
conductances, traces, weights and all integer state.  Two allowances, both
written here:
* outputs that go through tanhf or expf (rate encoding and its variants,
  oscillator, som, nvm) compare with relative tolerance 1e-5, and so do the
  values those outputs feed back into: the nvm case's state, inputs and
  recurrently learned weights, and the structures case's oscillator weights,
  state and bold.  The host C library's tanhf is not correctly rounded, so no
  GPU evaluation reproduces it bit for bit;
* in fp32 arrays any two NaNs match (x86, Arm and the GPU each produce a
  different default NaN payload for 0/0).
"""
import pytest

from tests.golden.cases import CASES
from tests.harness import compare, float_like_keys, load_fixture, run_library, run_oracle

pytestmark = pytest.mark.gpu

RATE_KEYS = ("rec/s/one", "rec/s/div", "rec/d/rtree", "rec/p/sdiv", "rec/m/hb", "rec/o/osc",
             "rec/o/som", "rec/v/", "neuron/v/", "matrix/v_rec", "rec/ff/o", "rec/ff/bp",
             "matrix/f_o", "neuron/ff/o/", "matrix/f_od")
RATE_TOL = 1e-5


@pytest.fixture(scope="module")
def syngen():
    from synaptogenesis_gb300 import syngen as sg
    assert sg.get_gpus(), "no CUDA GPU visible"
    return sg


@pytest.mark.parametrize("name", sorted(CASES))
def test_library_matches_reference_fixture(syngen, name):
    case = CASES[name]
    got = run_library(case, syngen)
    problems = compare(got, load_fixture(name), tol=RATE_TOL, float_keys=RATE_KEYS,
                       nan_keys=float_like_keys(case))
    assert not problems, problems


@pytest.mark.parametrize("path", ["tma", "small"])
@pytest.mark.parametrize("name", ["iz_c0_8", "iz_c0_32", "iz_opcodes", "iz_plastic",
                                  "iz_subset_columns"])
def test_izhikevich_matrix_activator_paths(syngen, name, path, monkeypatch):
    """Fully connected and subset Izhikevich connections take the TMA pipeline
    or, for few source rows, the one-pass kernel; each path alone matches the
    reference's fixture."""
    monkeypatch.setenv("SG_IZ_COLS_PATH", path)
    case = CASES[name]
    got = run_library(case, syngen)
    problems = compare(got, load_fixture(name), nan_keys=float_like_keys(case))
    assert not problems, problems


@pytest.mark.parametrize("name", ["iz_c0_32", "iz_plastic", "gol_16x16"])
def test_library_matches_oracle_longer(syngen, name):
    case = CASES[name]
    steps = 2 * case.steps
    got = run_library(case, syngen, steps=steps)
    want = run_oracle(case, steps=steps)
    problems = compare(got, want, nan_keys=float_like_keys(case))
    assert not problems, problems


def test_plastic_short_term_fixed_points_match_oracle(syngen):
    """The plastic case with half the synapses at the short-term fixed points
    (w = U = 0.5 for "add" connections, R = 1), where the updater skips the
    unchanged short-term values: bit-exact against the oracle."""
    import copy

    import numpy as np

    from tests.golden.cases import Case
    base = CASES["iz_plastic"]

    def inject(rng, sizes):
        d = base.inject(rng, sizes)
        pick = np.random.default_rng(5)
        for key in list(d):
            if key[0] == "matrix" and key[2] == "short term w":
                arr = d[key].copy()
                arr[pick.random(arr.size) < 0.5] = np.float32(0.5)
                d[key] = arr
        return d

    case = Case("iz_plastic_fixed_points", copy.deepcopy(base.net), 200, base.seed, inject=inject,
                inputs=base.inputs, record=base.record, final=base.final, tol=base.tol)
    got = run_library(case, syngen)
    want = run_oracle(case)
    problems = compare(got, want, nan_keys=float_like_keys(case))
    assert not problems, problems


@pytest.mark.parametrize("overlap", [True, False])
def test_overlapped_learning_matches_oracle(syngen, overlap):
    """Learning on the engine's second stream, overlapping the next step's
    activations (the default for large plastic networks), forced on and off
    for the plastic case: bit-exact against the oracle either way."""
    case = CASES["iz_plastic"]
    steps = 2 * case.steps
    got = run_library(case, syngen, steps=steps, extra_args={"overlap learning": overlap})
    want = run_oracle(case, steps=steps)
    problems = compare(got, want, nan_keys=float_like_keys(case))
    assert not problems, problems


@pytest.mark.parametrize("graphs", [True, False])
@pytest.mark.parametrize("name", ["dendrites", "second_order", "sparse"])
def test_cases_without_environment(syngen, name, graphs):
    """The dendritic-tree, second-order and sparse cases with no I/O modules
    (so the engine captures its steps in CUDA graphs, or not), their source
    layers driven by flat init configs: bit-exact against the oracle over
    twice the fixture's steps, rate_encoding outputs within RATE_TOL (tanhf)."""
    import copy

    from tests.golden.cases import Case
    base = CASES[name]
    net = copy.deepcopy(base.net)
    k = 0
    for st in net["structures"]:
        for layer in st["layers"]:
            if layer["name"] in base.inputs:
                layer["init config"] = {"type": "flat", "value": 0.5 + 0.25 * k}
                k += 1
    final = list(base.final) + [("neuron", s, l, "output") for (s, l) in base.record]
    case = Case(name + "_no_env", net, 2 * base.steps, base.seed, inject=base.inject, final=final)
    got = run_library(case, syngen, extra_args={"graphs": graphs})
    want = run_oracle(case)
    problems = compare(got, want, tol=RATE_TOL,
                       float_keys=("neuron/d/rtree/output", "neuron/p/sdiv/output"),
                       nan_keys=float_like_keys(case))
    assert not problems, problems


def test_reference_state_continues_here(syngen, tmp_path):
    """State interchange on the GPU: the plastic case's state saved by the
    reference's library after 75 of the fixture's 150 steps (a state file in
    the reference's record format), loaded here and run for the remaining 75
    steps, gives the reference's spike records of those steps and its final
    state, bit for bit."""
    import numpy as np
    from tests.harness import GOLDEN
    case = CASES["iz_plastic"]
    with np.load(GOLDEN + "/iz_plastic_state75.npz") as z:
        path = tmp_path / "reference.state"
        path.write_bytes(z["state"].tobytes())
    got = run_library(case, syngen, steps=75, state_file=str(path), start=75)
    want = load_fixture("iz_plastic")
    want = {k: (v[75:] if k.startswith("rec/") else v) for k, v in want.items()}
    problems = compare(got, want, nan_keys=float_like_keys(case))
    assert not problems, problems
