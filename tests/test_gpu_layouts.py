"""GPU test of the device layouts of per-synapse arrays: values written into
the host mirrors of a fully connected matrix (banded on the device, with a
row count that is not a multiple of the band), a subset matrix and a
convergent matrix (transposed on the device) come back unchanged after
uploads, runs without learning and downloads -- the conversions run as
device kernels."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    from synaptogenesis_gb300 import syngen
    assert syngen.get_gpus(), "no CUDA GPU visible"
    syngen.set_warnings(False)
    return syngen


def test_matrix_layouts_round_trip(sg):
    net_dict = {"structures": [{"name": "s", "type": "parallel", "layers": [
        {"name": "a", "neural model": "izhikevich", "rows": 13, "columns": 7},
        {"name": "b", "neural model": "izhikevich", "rows": 5, "columns": 11},
        {"name": "c", "neural model": "izhikevich", "rows": 9, "columns": 9}]}],
        "connections": [
            {"name": "fc", "from layer": "a", "to layer": "b", "type": "fully connected",
             "opcode": "add", "plastic": False, "delay": 2,
             "weight config": {"type": "random", "max weight": 0.5, "seed": 3}},
            {"name": "sub", "from layer": "a", "to layer": "c", "type": "subset", "opcode": "sub",
             "plastic": False,
             "subset config": {"from row start": 1, "from row end": 12, "from column start": 0,
                               "from column end": 7, "to row start": 2, "to row end": 9,
                               "to column start": 1, "to column end": 6},
             "weight config": {"type": "random", "max weight": 0.5, "seed": 4}},
            {"name": "conv", "from layer": "c", "to layer": "a", "type": "convergent",
             "opcode": "add", "plastic": False,
             "weight config": {"type": "random", "max weight": 0.5, "seed": 5},
             "arborized config": {"field size": 3, "stride": 1, "wrap": True}}]}
    net = sg.Network(net_dict)
    net.build_state()
    rng = np.random.default_rng(9)
    want = {}
    for cname in ("fc", "sub", "conv"):
        for key in ("weights", "short term w", "short term R", "long trace"):
            arr = net.get_weight_matrix(cname, key).to_np_array()
            vals = rng.uniform(0.0, 1.0, arr.size).astype(np.float32)
            arr.view(np.float32)[:] = vals
            want[(cname, key)] = vals
    # runs without learning move the state to the device and back; weights and
    # short-term factors are read-only there (the traces change)
    for steps in (1, 3):
        rep = net.run(sg.Environment({"modules": []}), {"iterations": steps, "learning flag": False})
        assert rep.obj is not None, sg.last_error()
        for (cname, key), vals in want.items():
            if key == "long trace":
                continue
            got = net.get_weight_matrix(cname, key).to_np_array().view(np.float32)
            assert np.array_equal(got, vals), (cname, key, steps)
