"""The bounded waits of the TMA activator (fully connected and subset
Izhikevich connections): with a testing hook the producer issues no loads for
one chunk, so the consumers' wait for it runs out.  Every wait in the kernel
has an iteration limit, the loads already issued are waited for before the
kernel ends, and the host reports the timeout as the run's error; the next
run, with the hook off, succeeds, and a fresh network still matches the
reference's fixture."""
import ctypes

import pytest

from tests.golden.cases import CASES
from tests.harness import compare, float_like_keys, load_fixture, run_library

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    from synaptogenesis_gb300 import syngen
    assert syngen.get_gpus(), "no CUDA GPU visible"
    syngen.set_warnings(False)
    return syngen


def test_tma_wait_timeout_is_reported(sg, monkeypatch):
    monkeypatch.setenv("SG_IZ_COLS_PATH", "tma")     # this case's rows would take the one-pass kernel
    lib = ctypes.CDLL(sg.LIB_PATH)
    lib.sg_test_cols_skip_chunk.argtypes = (ctypes.c_int,)
    lib.sg_test_cols_skip_chunk.restype = ctypes.c_bool
    case = CASES["iz_subset_columns"]      # q_in: 192 source rows, 6 chunks of 32
    net = sg.Network(case.net)
    net.build_state()
    env = sg.Environment({"modules": []})
    args = {"iterations": 1, "learning flag": False, "graphs": False}
    assert net.run(env, dict(args)).obj is not None, sg.last_error()
    try:
        assert lib.sg_test_cols_skip_chunk(2)
        rep = net.run(env, dict(args))
        assert rep is None or rep.obj is None
        assert "timed out" in sg.last_error()
    finally:
        assert lib.sg_test_cols_skip_chunk(-1)
    rep = net.run(env, dict(args))
    assert rep is not None and rep.obj is not None, sg.last_error()
    got = run_library(case, sg)
    assert not compare(got, load_fixture(case.name), nan_keys=float_like_keys(case))
