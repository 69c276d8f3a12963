"""The drop-in claim: the reference's own, unmodified lib/syngen.py binds this
library (it loads `libsyngen.so` by name; the library carries that soname and
its build folder goes on LD_LIBRARY_PATH) and drives the fixture cases through
it.  Without a GPU the cases are built, injected, saved, reloaded and read
back, and a run fails cleanly; with one they run and match the fixtures
recorded from the reference's own library.  Needs the reference checkout."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def reference_available():
    from oracle import build_ref
    return os.path.isfile(os.path.join(build_ref.reference_root(), "lib", "syngen.py"))


@pytest.mark.skipif(not reference_available(), reason="the reference checkout is needed")
def test_reference_frontend_binds_this_library(tmp_path):
    from synaptogenesis_gb300 import build
    lib = build.build()
    env = dict(os.environ, LD_LIBRARY_PATH=os.path.dirname(lib) + ":" +
               os.environ.get("LD_LIBRARY_PATH", ""))
    env.pop("SYNGEN_LIB", None)
    out = tmp_path / "r.json"
    r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "golden",
                                                     "ref_frontend_check.py"), str(out)],
                       env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(out.read_text())
    assert res["bound_library"] == "gb300"
    for name, c in res["cases"].items():
        if res["gpu"]:
            assert c["run_matches_fixture"], (name, c["problems"])
        else:
            assert c["state_round_trip"], name
            assert c["run_without_gpu_fails_cleanly"], name
