"""State files interchange with the reference (src/core/state/state.cpp:365-447):
a state the reference's own CPU library saved after running a case loads into
this library with every array equal, and a state this library saved loads
into the reference with every array equal.  Records are [owner hash, variable
hash, bytes][data] with std::hash keys; both sides skip records they do not
hold.  The reference runs in a child process (tests/golden/ref_state.py), and
these checks need its checkout; the GPU test (test_gpu_golden) continues a
reference-saved state on the GPU."""
import os
import subprocess
import sys

import numpy as np
import pytest

from tests.golden.cases import CASES, callback_injections
from tests.golden.ref_state import state_keys
from tests.harness import case_sizes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASE_NAMES = ["iz_plastic", "base_all_types", "gol_16x16", "iz_subset_columns", "dendrites"]


def reference_available():
    from oracle import build_ref
    return os.path.isdir(os.path.join(build_ref.reference_root(), "src"))


pytestmark = pytest.mark.skipif(not reference_available(),
                                reason="the reference checkout is needed to run it")


def run_reference(*args):
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "golden", "ref_state.py")]
                       + [str(a) for a in args], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]


def ours(case, inject):
    """The case's network built by this library (no run: no GPU needed),
    with the case's injections applied when `inject`."""
    from synaptogenesis_gb300 import syngen as sg
    sizes = case_sizes(case)
    net_dict, injections, weight_arrays, delay_arrays = callback_injections(
        case.net, case.injections(sizes))
    sg.create_weight_callback("golden_weight",
                              lambda ID, size, w: sg.FloatArray(size, w).to_np_array().__setitem__(
                                  slice(None), weight_arrays[ID]))
    sg.create_delay_weight_callback("golden_delay",
                                    lambda ID, size, w, d: sg.IntArray(size, d).to_np_array()
                                    .__setitem__(slice(None), delay_arrays[ID]))
    net = sg.Network(net_dict)
    net.build_state()
    if inject:
        for key, arr in injections.items():
            if key[0] == "neuron":
                dst = net.get_neuron_data(key[1], key[2], key[3]).to_np_array()
            else:
                dst = net.get_weight_matrix(key[1], key[2]).to_np_array()
            dst.view(arr.dtype)[:] = arr
    return net


def arrays(net, case):
    out = {}
    for key in state_keys(case):
        if key[0] == "neuron":
            a = net.get_neuron_data(key[1], key[2], key[3])
        else:
            a = net.get_weight_matrix(key[1], key[2])
        a = np.array(a.to_np_array(), copy=True)
        out["/".join(key)] = a.view(np.uint32) if a.dtype == np.float32 else a
    return out


def same(got, want):
    problems = []
    for k, w in want.items():
        g = got[k]
        if g.shape != w.shape or not np.array_equal(g, w):
            problems.append(k)
    return problems


@pytest.mark.parametrize("name", CASE_NAMES)
def test_reference_state_loads_here(tmp_path, name):
    case = CASES[name]
    state, dumped = tmp_path / "ref.state", tmp_path / "ref.npz"
    run_reference("save", name, 20, state, dumped)
    net = ours(case, inject=False)
    net.load_state(str(state))
    with np.load(dumped) as z:
        want = {k: z[k] for k in z.files}
    assert not same(arrays(net, case), want)


@pytest.mark.parametrize("name", CASE_NAMES)
def test_state_saved_here_loads_in_reference(tmp_path, name):
    case = CASES[name]
    net = ours(case, inject=True)
    state, dumped = tmp_path / "ours.state", tmp_path / "ref.npz"
    net.save_state(str(state))
    run_reference("load", name, state, dumped)
    with np.load(dumped) as z:
        got = {k: z[k] for k in z.files}
    assert not same(got, arrays(net, case))


def test_size_mismatch_is_an_error(tmp_path):
    """A record whose owner and variable match but whose size does not (the
    reference would resize the array) is refused with a message."""
    from synaptogenesis_gb300 import syngen as sg
    case = CASES["gol_16x16"]
    net = ours(case, inject=True)
    path = tmp_path / "s.state"
    net.save_state(str(path))
    raw = bytearray(path.read_bytes())
    # first record: [hash, type, bytes]; claim 4 bytes more, append them
    n = int.from_bytes(raw[16:24], "little")
    raw[16:24] = (n + 4).to_bytes(8, "little")
    raw[24 + n:24 + n] = bytes(4)
    path.write_bytes(bytes(raw))
    assert not sg._syn.load_state(net.state, str(path).encode())
    assert "bytes" in sg.last_error()
