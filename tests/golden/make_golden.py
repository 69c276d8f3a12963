"""Generate golden fixtures by running the reference's own CPU library.

Usage (in a checkout that has the reference sources):
    python oracle/build_ref.py
    OMP_NUM_THREADS=1 python tests/golden/make_golden.py [case ...]
    OMP_NUM_THREADS=1 python tests/golden/make_golden.py c0_1000 c2_1000
    python tests/golden/make_golden.py c1_10000      # game_of_life: any thread count

The configurations at their stated sizes (c0_1000, c1_10000, c2_1000) are
recorded as digests (see configs.py); the other cases as whole arrays.

The reference library (oracle/_ref/libsyngen.so, built from the reference
sources by oracle/build_ref.py) is driven through the reference's own Python
front-end (lib/syngen.py of the reference checkout).  Every random quantity is
injected from the seeds in cases.py; the reference's recorded outputs are
written to tests/golden/<case>.npz.  One OpenMP thread is used because the
reference's time-since-spike update is order dependent (it races with more).
"""
import copy
import ctypes
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from cases import CASES, callback_injections  # noqa: E402


def load_reference_syngen():
    from oracle import build_ref
    lib = build_ref.build()
    ctypes.CDLL(lib, mode=ctypes.RTLD_GLOBAL)   # satisfies CDLL('libsyngen.so')
    path = os.path.join(build_ref.reference_root(), "lib", "syngen.py")
    spec = importlib.util.spec_from_file_location("ref_syngen", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.set_warnings(False)
    mod.set_suppress_output(False)
    return mod


from tests.harness import case_sizes  # noqa: E402  (sizes checked against the reference below)


def run_case(sg, case):
    sizes = case_sizes(case)
    # Delays are not a readable/writable weight-matrix variable in the
    # reference, and a sparse connection's dense weights exist only while its
    # state is built: both go in through weight-config callbacks.
    net_dict, injections, weight_arrays, delay_arrays = callback_injections(
        case.net, case.injections(sizes))

    def weight_cb(ID, size, weights):
        arr = weight_arrays[ID]
        assert size == arr.size
        sg.FloatArray(size, weights).to_np_array()[:] = arr

    def delay_cb(ID, size, weights, delays):
        arr = delay_arrays[ID]
        assert size == arr.size
        sg.IntArray(size, delays).to_np_array()[:] = arr

    sg._delay_weight_callbacks = {}     # the reference front-end never defines it
    if not hasattr(sg, "_weight_callbacks"):
        sg._weight_callbacks = {}
    sg.create_weight_callback("golden_weight", weight_cb)
    sg.create_delay_weight_callback("golden_delay", delay_cb)
    net = sg.Network(net_dict)
    net.build_state()
    for c in case.net["connections"]:
        if c.get("sparse"):
            continue
        got = net.get_weight_matrix(c["name"], "weights").size
        assert got == sizes["conn:" + c["name"]], (c["name"], got)
    for key, arr in injections.items():
        if key[0] == "neuron":
            dst = net.get_neuron_data(key[1], key[2], key[3]).to_np_array()
        else:
            dst = net.get_weight_matrix(key[1], key[2]).to_np_array()
        assert dst.size == arr.size, (key, dst.size, arr.size)
        dst.view(arr.dtype)[:] = arr
    inputs = case.input_arrays(sizes)

    step = {"in": 0}
    in_layers = sorted(case.inputs)
    rec = {k: [] for k in case.record}

    def in_cb(ID, size, ptr):
        name = in_layers[ID]
        sg.FloatArray(size, ptr).to_np_array()[:] = inputs[step["in"]][name]
        if ID == len(in_layers) - 1:
            step["in"] += 1

    def out_cb(ID, size, ptr):
        rec[case.record[ID]].append(
            sg.FloatArray(size, ptr).to_np_array().view(np.uint32).copy())

    sg.create_io_callback("golden_in", in_cb)
    sg.create_io_callback("golden_out", out_cb)
    modules = []
    if in_layers:
        modules.append({"type": "callback", "layers": [
            {"structure": _struct_of(case, l), "layer": l, "input": True,
             "function": "golden_in", "id": i} for i, l in enumerate(in_layers)]})
    if case.record:
        modules.append({"type": "callback", "layers": [
            {"structure": s, "layer": l, "output": True, "function": "golden_out", "id": i}
            for i, (s, l) in enumerate(case.record)]})
    report = net.run(sg.Environment({"modules": modules}),
                     {"iterations": case.steps, "multithreaded": False, "worker threads": 0,
                      "learning flag": case.learning})
    assert report is not None
    out = {}
    for (s, l), frames in rec.items():
        assert len(frames) == case.steps, (s, l, len(frames))
        out["rec/%s/%s" % (s, l)] = np.stack(frames)
    for key in case.final:
        if key[0] == "neuron":
            arr = net.get_neuron_data(key[1], key[2], key[3])
            name = "neuron/%s/%s/%s" % key[1:]
        else:
            arr = net.get_weight_matrix(key[1], key[2])
            name = "matrix/%s/%s" % key[1:]
        a = arr.to_np_array().copy()
        out[name] = a.view(np.uint32) if a.dtype == np.float32 else a
    return out


def _struct_of(case, layer):
    for st in case.net["structures"]:
        for l in st["layers"]:
            if l["name"] == layer:
                return st["name"]
    raise KeyError(layer)


def scale_fixture(sg, name):
    """Digest fixtures of the configurations at their stated sizes
    (tests/golden/configs.py): per-step output digests and spike counts, and
    state digests after 100 steps and at the end."""
    from tests.golden import configs
    from tests.harness import run_digest, run_gol_digest
    if name == "c1_10000":
        return run_gol_digest(sg, 2048, 10000, 1000)
    case = {"c0_1000": configs.c0_case, "c2_1000": configs.c2_case}[name]()
    return run_digest(case, sg, checkpoints=configs.CHECKPOINTS)


SCALE = ("c0_1000", "c1_10000", "c2_1000")


def state_fixture(name):
    """``<case>_state<steps>``: the state file the reference saves after
    running the case for that many steps (bytes), for the GPU test that
    continues it here."""
    import subprocess
    import tempfile
    case, steps = name.rsplit("_state", 1)
    with tempfile.TemporaryDirectory() as d:
        state, dumped = os.path.join(d, "s.state"), os.path.join(d, "s.npz")
        env = dict(os.environ, OMP_NUM_THREADS="1")
        subprocess.run([sys.executable, os.path.join(HERE, "ref_state.py"), "save", case, steps,
                        state, dumped], env=env, check=True)
        with open(state, "rb") as f:
            return {"state": np.frombuffer(f.read(), np.uint8)}


def main(names):
    sg = load_reference_syngen()
    for name in names or sorted(CASES):
        if "_state" in name:
            out = state_fixture(name)
            path = os.path.join(HERE, name + ".npz")
            np.savez_compressed(path, **out)
            print("wrote", path)
            continue
        if name in SCALE:
            out = scale_fixture(sg, name)
            path = os.path.join(HERE, name + ".npz")
            np.savez_compressed(path, **out)
            print("wrote", path, sum(v.nbytes for v in out.values()), "bytes")
            continue
        out = run_case(sg, CASES[name])
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **out)
        print("wrote", path, sum(v.nbytes for v in out.values()), "bytes")


if __name__ == "__main__":
    main(sys.argv[1:])
