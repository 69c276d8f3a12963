"""GPU parity: every golden case through the C-ABI against the reference's own
recorded results (bit-exact), and against the oracle.

Bit-exact: spike rasters, output-history words, voltages, recoveries,
conductances, traces, weights and all integer state.  The only tolerance is
for rate_encoding outputs, which go through tanhf (the GPU's tanhf and the
host C library's may differ in the last bit): relative 1e-5.
"""
import pytest

from tests.golden.cases import CASES
from tests.harness import compare, load_fixture, run_library, run_oracle

pytestmark = pytest.mark.gpu

RATE_KEYS = ("rec/s/one", "rec/s/div")


@pytest.fixture(scope="module")
def syngen():
    from synaptogenesis_gb300 import syngen as sg
    assert sg.get_gpus(), "no CUDA GPU visible"
    return sg


@pytest.mark.parametrize("name", sorted(CASES))
def test_library_matches_reference_fixture(syngen, name):
    got = run_library(CASES[name], syngen)
    problems = compare(got, load_fixture(name), tol=1e-5, float_keys=RATE_KEYS)
    assert not problems, problems


@pytest.mark.parametrize("name", ["iz_c0_32", "iz_plastic"])
def test_library_matches_oracle_longer(syngen, name):
    case = CASES[name]
    steps = 2 * case.steps
    got = run_library(case, syngen, steps=steps)
    want = run_oracle(case, steps=steps)
    problems = compare(got, want)
    assert not problems, problems
