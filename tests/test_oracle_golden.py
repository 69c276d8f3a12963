"""The CPU oracle against fixtures recorded from the reference's own CPU path.

This pins the oracle: every case is bit-exact (spike rasters, output history
words, voltages, traces, weights) against what the reference produced on the
same injected inputs.
"""
import pytest

from tests.golden.cases import CASES
from tests.harness import compare, float_like_keys, load_fixture, run_oracle


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_fixture(name):
    problems = compare(run_oracle(CASES[name]), load_fixture(name),
                       nan_keys=float_like_keys(CASES[name]))
    assert not problems, problems
