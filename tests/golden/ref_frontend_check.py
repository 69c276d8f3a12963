"""Drives this library through the reference's own, unmodified front-end
(lib/syngen.py of the reference checkout), which loads `libsyngen.so` by
name: the parent test starts this script with the library's build folder on
LD_LIBRARY_PATH, so that name resolves to this library.

  python tests/golden/ref_frontend_check.py <out.json>

For the fixture cases iz_c0_8, gol_16x16 and iz_plastic it builds the network
through the reference's front-end, applies the case's injections through its
getters (weights and delays through its weight callbacks), saves and reloads
the state, and reads every compared array back.  With a GPU it also runs each
case and compares the recorded outputs and final arrays with the fixture
(recorded from the reference's own library); without one it checks that the
run fails cleanly.  The results go to <out.json>.
"""
import importlib.util
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_ref  # noqa: E402
from tests.golden.cases import CASES  # noqa: E402
from tests.harness import compare, float_like_keys, load_fixture, run_library  # noqa: E402


def load_reference_frontend():
    path = os.path.join(build_ref.reference_root(), "lib", "syngen.py")
    spec = importlib.util.spec_from_file_location("reference_syngen", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.set_warnings(False)
    mod._delay_weight_callbacks = {}     # the reference front-end never defines it
    return mod


def main(out_path):
    sg = load_reference_frontend()
    result = {"bound_library": None, "cases": {}}
    # only this library exports the sg_* extensions
    result["bound_library"] = "gb300" if hasattr(sg._syn, "sg_version") else "other"
    has_gpu = len(sg.get_gpus()) > 0
    result["gpu"] = has_gpu
    for name in ("iz_c0_8", "gol_16x16", "iz_plastic"):
        case = CASES[name]
        r = {}
        if has_gpu:
            got = run_library(case, sg)
            problems = compare(got, load_fixture(name), nan_keys=float_like_keys(case))
            r["run_matches_fixture"] = not problems
            r["problems"] = problems[:3]
        else:
            # build, inject, save, reload and read back; a run must fail cleanly
            net = sg.Network(case.net)
            net.build_state()
            w = net.get_weight_matrix(case.net["connections"][0]["name"], "weights").to_np_array()
            w[:] = np.arange(w.size, dtype=np.float32)
            with tempfile.TemporaryDirectory() as d:
                path = os.path.join(d, "s.state")
                net.save_state(path)
                w[:] = 0.0
                net.load_state(path)
            back = net.get_weight_matrix(case.net["connections"][0]["name"], "weights").to_np_array()
            r["state_round_trip"] = bool(np.array_equal(back, np.arange(back.size, dtype=np.float32)))
            report = net.run(sg.Environment({"modules": []}), {"iterations": 1})
            r["run_without_gpu_fails_cleanly"] = report is None or getattr(report, "obj", None) is None
        result["cases"][name] = r
    with open(out_path, "w") as f:
        json.dump(result, f)


if __name__ == "__main__":
    main(sys.argv[1])
