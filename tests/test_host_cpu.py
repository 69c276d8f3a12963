"""CPU tests of the library's host side (no GPU needed: device memory is only
allocated when a run starts).

* the C-ABI library loads and exports every function include/syngen.h declares;
* building a state reproduces the oracle's initial state exactly (Izhikevich
  resting state, distance-based delays, short-term-plasticity defaults, ...);
* schema quirks and error behaviour of the reference;
* JSON, property and state round trips.
"""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def sg():
    from synaptogenesis_gb300 import build
    build.build()
    from synaptogenesis_gb300 import syngen
    syngen.set_warnings(False)
    return syngen


def header_functions():
    text = open(os.path.join(ROOT, "include", "syngen.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w\s\*]*?\b(\w+)\s*\([^;]*\)\s*;", text, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "while")))


def test_library_exports_every_header_function(sg):
    lib = ctypes.CDLL(sg.LIB_PATH)
    names = header_functions()
    assert len(names) >= 60
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


@pytest.mark.parametrize("name", ["iz_opcodes", "iz_plastic", "base_all_types", "iz_c0_8",
                                  "gol_two_word_history", "dendrites", "second_order", "sparse",
                                  "models", "spnet", "oscillator_som", "nvm", "structures"])
def test_initial_state_matches_oracle(sg, name):
    from oracle.oracle import OracleNetwork
    from tests.golden.cases import CASES
    case = CASES[name]
    net = sg.Network(case.net)
    net.build_state()
    assert net.state, sg.last_error()
    onet = OracleNetwork(case.net)
    for l in onet.layers:
        for k, v in onet.neuron[l].items():
            got = net.get_neuron_data(l.structure, l.name, k).to_np_array()
            assert np.array_equal(got.view(np.uint32), v.view(np.uint32)), (l.name, k)
    for c in onet.conns:
        for k, v in onet.matrix[c].items():
            got = net.get_weight_matrix(c.name, k).to_np_array()
            assert got.size == v.size or k == "time since spike", (c.name, k)
            if k != "weights":
                assert np.array_equal(got.view(np.uint32)[:v.size], v.view(np.uint32)), (c.name, k)


def test_sparse_compaction_matches_oracle(sg):
    """Sparse connections compacted from dense weights set by a weight
    callback: every per-synapse array (compacted weights, distance delays
    with their -1 padding, Izhikevich variables) equals the oracle's."""
    from oracle.oracle import OracleNetwork
    from tests.golden.cases import CASES, callback_injections
    from tests.harness import case_sizes
    case = CASES["sparse"]
    net_dict, _, weights, _ = callback_injections(
        case.net, {k: v for k, v in case.injections(case_sizes(case)).items()
                   if k[2] == "init weights"})

    def weight_cb(ID, size, ptr):
        sg.FloatArray(size, ptr).to_np_array()[:] = weights[ID]

    sg.create_weight_callback("golden_weight", weight_cb)
    net = sg.Network(net_dict)
    net.build_state()
    assert net.state, sg.last_error()
    onet = OracleNetwork(net_dict, weight_callbacks={
        "golden_weight": lambda ID, w: w.__setitem__(slice(None), weights[ID])})
    for c in onet.conns:
        for k, v in onet.matrix[c].items():
            got = net.get_weight_matrix(c.name, k).to_np_array()
            n = v.size if k == "time since spike" else got.size
            assert got.size == v.size or k == "time since spike", (c.name, k, got.size, v.size)
            assert np.array_equal(got.view(np.uint32)[:n], v.view(np.uint32)[:n]), (c.name, k)
    assert onet.connection("p_zero").num_weights == 48          # one synapse per destination
    assert onet.connection("i_rec").kmax < 25


def _randomized_net():
    """One-to-one, convergent and divergent randomized projections (relay and
    Izhikevich targets, clipped and wrapping fields), seeded."""
    return {"structures": [{"name": "s", "layers": [
        {"name": "a", "neural model": "relay", "rows": 6, "columns": 6},
        {"name": "b", "neural model": "relay", "rows": 6, "columns": 6},
        {"name": "iz", "neural model": "izhikevich", "rows": 6, "columns": 6},
        {"name": "c", "neural model": "relay", "rows": 3, "columns": 3}]}],
        "connections": [
            {"name": "r1", "from layer": "a", "to layer": "b", "type": "one to one",
             "randomized projection": True, "plastic": False,
             "weight config": {"type": "flat", "weight": 0.5, "seed": 5}},
            {"name": "r2", "from layer": "a", "to layer": "b", "type": "convergent",
             "randomized projection": True, "plastic": False,
             "arborized config": {"field size": 3, "wrap": False},
             "weight config": {"type": "flat", "weight": 0.25, "seed": 6}},
            {"name": "r3", "from layer": "a", "to layer": "iz", "type": "convergent",
             "randomized projection": True, "plastic": False,
             "arborized config": {"field size": 3, "wrap": True},
             "weight config": {"type": "flat", "weight": 0.5, "seed": 7}},
            {"name": "r4", "from layer": "c", "to layer": "b", "type": "divergent",
             "randomized projection": True, "plastic": False,
             "arborized config": {"field size": 3, "stride": 2, "wrap": True},
             "weight config": {"type": "flat", "weight": 0.75, "seed": 8}},
            {"name": "r5", "from layer": "c", "to layer": "iz", "type": "divergent",
             "randomized projection": True, "plastic": False,
             "arborized config": {"field size": 3, "stride": 2, "wrap": False},
             "weight config": {"type": "flat", "weight": 0.5, "seed": 9}}]}


def test_randomized_projection_state_matches_oracle(sg):
    """Randomized projections (seeded draws; the reference's are unseeded):
    the compacted weights and the distance delays of the randomized sources
    equal the oracle's, and the sources really moved."""
    from oracle.oracle import OracleNetwork
    net = _randomized_net()
    n = sg.Network(net)
    n.build_state()
    assert n.state, sg.last_error()
    o = OracleNetwork(net)
    for c in o.conns:
        for k, v in o.matrix[c].items():
            got = n.get_weight_matrix(c.name, k).to_np_array()
            m = min(got.size, v.size)
            assert np.array_equal(got.view(np.uint32)[:m], v.view(np.uint32)[:m]), (c.name, k)
    r1 = o.connection("r1")
    assert not np.array_equal(r1.from_idx[:r1.nvisits], np.arange(36))


def test_randomized_projection_outside_a_non_square_layer_is_refused(sg):
    """The convergent form's row pitch (the source's row count) indexes past
    a 6x5 source layer: refused at build instead of reading outside it."""
    from oracle.oracle import OracleNetwork
    net = _randomized_net()
    for l in net["structures"][0]["layers"]:
        l["columns"] = 5
    net["connections"] = [net["connections"][1]]
    n = sg.Network(net)
    n.build_state()
    assert n.state is None and "outside the source layer" in sg.last_error()
    with pytest.raises(ValueError, match="outside the source layer"):
        OracleNetwork(net)


@pytest.mark.parametrize("conn", [
    {"type": "fully connected"}, {"type": "subset"},
    {"type": "convergent", "convolutional": True, "arborized config": {"field size": 3}}])
def test_randomized_projection_errors(sg, conn):
    net = _randomized_net()
    bad = dict(net["connections"][0], **conn)
    if conn["type"] == "subset":
        bad["subset config"] = {"from row end": 2, "from column end": 2, "to row end": 2, "to column end": 2}
    net["connections"] = [bad]
    n = sg.Network(net)
    assert n.obj is None and "randomize projection" in sg.last_error()


def test_column_offset_quirk_and_weight_counts(sg):
    from oracle.oracle import OracleNetwork
    net = {"structures": [{"name": "s", "layers": [
        {"name": "a", "neural model": "relay", "rows": 7, "columns": 9},
        {"name": "b", "neural model": "relay", "rows": 5, "columns": 6}]}],
        "connections": [
            {"name": "co", "from layer": "a", "to layer": "b", "type": "convergent",
             "arborized config": {"row field size": 3, "column field size": 2,
                                  "column offset": -3, "stride": 1}},
            {"name": "dv", "from layer": "b", "to layer": "a", "type": "divergent",
             "arborized config": {"field size": 3, "stride": 2}},
            {"name": "ss", "from layer": "a", "to layer": "b", "type": "subset",
             "subset config": {"from row start": 1, "from row end": 4, "from column start": 0,
                               "from column end": 2, "to row start": 2, "to row end": 5,
                               "to column start": 3, "to column end": 6}}]}
    n = sg.Network(net)
    n.build_state()
    o = OracleNetwork(net)
    for c in o.conns:
        assert n.get_weight_matrix(c.name).size == c.num_weights
    # "column offset" alone is ignored (read from "row offset"): it is 0, not -3.
    assert o.connection("co").c.col_offset == 0


@pytest.mark.parametrize("bad", [
    {"structures": [{"name": "s", "layers": [{"name": "a", "neural model": "nope", "rows": 2, "columns": 2}]}]},
    {"structures": [{"name": "s", "layers": [{"name": "a", "neural model": "relay", "rows": 0, "columns": 2}]}]},
    {"structures": [{"name": "s", "layers": [
        {"name": "a", "neural model": "relay", "rows": 2, "columns": 2},
        {"name": "b", "neural model": "relay", "rows": 3, "columns": 2}]}],
     "connections": [{"from layer": "a", "to layer": "b", "type": "one to one"}]},
    {"structures": [{"name": "s", "layers": [
        {"name": "a", "neural model": "relay", "rows": 2, "columns": 2}]}],
     "connections": [{"from layer": "a", "to layer": "a", "type": "convergent"}]},
])
def test_invalid_networks_fail_like_the_reference(sg, bad):
    n = sg.Network(bad)
    assert n.obj is None          # create_network returns nullptr
    assert sg.last_error()


def _dendrite_net(dendrites, conns, model="relay"):
    return {"structures": [{"name": "s", "layers": [
        {"name": "a", "neural model": "relay", "rows": 3, "columns": 3},
        {"name": "b", "neural model": "relay", "rows": 3, "columns": 3},
        {"name": "t", "neural model": model, "rows": 3, "columns": 3, "dendrites": dendrites}]}],
        "connections": conns}


_SO = [{"name": "g", "second order": True}]
_FC = {"from layer": "a", "to layer": "t", "type": "fully connected", "plastic": False}

# Each network breaks one rule of the reference's dendritic trees
# (layer.cpp:135-153, dendritic_node.cpp:80-140, connection.cpp:149-191).
DENDRITE_ERRORS = [
    ("Attempted to dendrite without name", _dendrite_net([{"opcode": "add"}], [])),
    ("Duplicate dendritic node name", _dendrite_net([{"name": "x"}, {"name": "x"}], [])),
    ("Duplicate dendritic node name", _dendrite_net([{"name": "root"}], [])),
    ("cannot have internal children",
     _dendrite_net([{"name": "g", "second order": True, "children": [{"name": "h"}]}], [])),
    ("Cannot find Dendritic Node", _dendrite_net([{"name": "x"}], [dict(_FC, dendrite="y")])),
    ("Plastic second order", _dendrite_net(_SO, [dict(_FC, dendrite="g", plastic=True)])),
    ("does not match host", _dendrite_net(_SO, [
        dict(_FC, dendrite="g"),
        {"from layer": "b", "to layer": "t", "type": "one to one", "plastic": False, "dendrite": "g"}])),
    ("must have fields that are the size of the input layer", _dendrite_net(_SO, [
        {"from layer": "a", "to layer": "t", "type": "convergent", "convolutional": True,
         "plastic": False, "dendrite": "g", "arborized config": {"field size": 3}},
        {"from layer": "b", "to layer": "t", "type": "convergent", "convolutional": True,
         "plastic": False, "dendrite": "g", "arborized config": {"field size": 3, "stride": 1}}])),
]


@pytest.mark.parametrize("message,net", DENDRITE_ERRORS)
def test_invalid_dendritic_trees_fail_like_the_reference(sg, message, net):
    from oracle.oracle import OracleNetwork
    n = sg.Network(net)
    assert n.obj is None and message in sg.last_error(), sg.last_error()
    with pytest.raises(ValueError, match=message):
        OracleNetwork(net)


def test_izhikevich_second_order_needs_direct_connections(sg):
    net = _dendrite_net(_SO, [dict(_FC, dendrite="g"), dict(_FC, dendrite="g")], model="izhikevich")
    n = sg.Network(net)
    n.build_state()
    assert n.state is None and "Unimplemented connection type" in sg.last_error()
    net = _dendrite_net(_SO, [dict(_FC, dendrite="g", direct=True), dict(_FC, dendrite="g", direct=True)],
                        model="izhikevich")
    n = sg.Network(net)
    n.build_state()
    assert n.state, sg.last_error()


def test_dendritic_registers_and_node_names(sg):
    """Registers follow the config's pre-order; each connection's name
    (its saved-state key) carries its node."""
    from oracle.oracle import OracleNetwork
    net = _dendrite_net([{"name": "p", "children": [{"name": "p1"}, {"name": "p2"}]}, {"name": "q"}],
                        [dict(_FC, dendrite="p2", name="c1"), dict(_FC, name="c0")])
    o = OracleNetwork(net)
    t = o.layer("t")
    assert [(d.name, d.reg) for d in t.dendrites()] == [("root", 0), ("p", 1), ("q", 4), ("p1", 2), ("p2", 3)]
    n = sg.Network(net)
    n.build_state()
    assert n.get_neuron_data("s", "t", "input").size == 5 * 9
    assert n.get_neuron_data("s", "a", "input").size == 9


def test_model_build_errors_match_the_reference(sg):
    """backprop_rate_encoding and sample build only in feedforward
    structures; the perceptron and som have no convolutional activator."""
    from oracle.oracle import OracleNetwork
    for model in ("backprop_rate_encoding", "sample"):
        net = {"structures": [{"name": "s", "layers": [
            {"name": "a", "neural model": model, "rows": 2, "columns": 2}]}]}
        n = sg.Network(net)
        n.build_state()
        assert n.state is None and "Cluster compatibility conflict" in sg.last_error()
        with pytest.raises(ValueError, match="Cluster compatibility"):
            OracleNetwork(net)
    net = {"structures": [{"name": "s", "layers": [
        {"name": "a", "neural model": "relay", "rows": 4, "columns": 4},
        {"name": "p", "neural model": "perceptron", "rows": 4, "columns": 4}]}],
        "connections": [{"from layer": "a", "to layer": "p", "type": "convergent",
                         "convolutional": True, "arborized config": {"field size": 3}}]}
    n = sg.Network(net)
    n.build_state()
    assert n.state is None and "Unimplemented connection type" in sg.last_error()
    net["structures"][0]["layers"][1]["neural model"] = "som"
    n = sg.Network(net)
    n.build_state()
    assert n.state is None and "Unimplemented connection type" in sg.last_error()
    with pytest.raises(ValueError, match="Unimplemented connection type"):
        OracleNetwork(net)


def _struct_net(kind, conns):
    return {"structures": [{"name": "s", "type": kind, "layers": [
        {"name": n, "neural model": "relay", "rows": 2, "columns": 2} for n in ("x", "a", "b")]}],
        "connections": [{"from layer": f, "to layer": t, "type": "one to one", "plastic": False,
                         "recurrent": r} for f, t, r in conns]}


@pytest.mark.parametrize("kind,conns,message", [
    ("sequential", [("x", "a", False), ("a", "b", False), ("b", "a", False)],
     "Sequential cluster failed to process all layers"),
    ("feedforward", [("x", "a", False), ("a", "b", False), ("b", "a", True)],
     "Feedforward engine requires a structure with no cycles"),
])
def test_structure_order_errors_match_the_reference(sg, kind, conns, message):
    """A sequential structure whose layers feed each other in a cycle (the
    reference loops forever there; here the walk stops with its error), and
    a feedforward structure with a cycle through a recurrent connection."""
    from oracle.oracle import OracleNetwork
    net = _struct_net(kind, conns)
    n = sg.Network(net)
    assert n.obj is None and message in sg.last_error(), sg.last_error()
    with pytest.raises(ValueError, match=message):
        OracleNetwork(net)


def test_sequential_order_follows_the_reference(sg):
    """Layers listed out of order step after the layers that feed them; a
    recurrent connection does not constrain the order."""
    from oracle.oracle import OracleNetwork
    net = _struct_net("sequential", [("b", "a", False), ("a", "x", False), ("x", "b", True)])
    o = OracleNetwork(net)
    assert [l.name for l in o.order["s"]] == ["b", "a", "x"]
    assert sg.Network(net).obj is not None


def test_izhikevich_gap_must_be_self_connection(sg):
    net = {"structures": [{"name": "s", "layers": [
        {"name": "a", "neural model": "izhikevich", "rows": 2, "columns": 2},
        {"name": "b", "neural model": "izhikevich", "rows": 2, "columns": 2}]}],
        "connections": [{"from layer": "a", "to layer": "b", "opcode": "gap"}]}
    n = sg.Network(net)
    n.build_state()
    assert n.state is None and "Gap junctions" in sg.last_error()


def test_large_distance_delays_are_rejected(sg):
    net = {"structures": [{"name": "s", "layers": [
        {"name": "a", "neural model": "izhikevich", "rows": 64, "columns": 64},
        {"name": "b", "neural model": "izhikevich", "rows": 64, "columns": 64}]}],
        "connections": [{"from layer": "a", "to layer": "b", "plastic": False}]}
    n = sg.Network(net)
    n.build_state()
    assert n.state is None and "delays cannot be greater than 31" in sg.last_error()


def test_weight_and_delay_callbacks(sg):
    seen = {}

    def wcb(ID, size, ptr):
        arr = sg.FloatArray(size, ptr).to_np_array()
        arr[:] = np.arange(size, dtype=np.float32) * (ID + 1)
        seen["w"] = size

    def dcb(ID, size, weights, delays):
        sg.IntArray(size, delays).to_np_array()[:] = np.arange(size) % 7
        seen["d"] = size

    sg.create_weight_callback("t_w", wcb)
    sg.create_delay_weight_callback("t_d", dcb)
    net = {"structures": [{"name": "s", "layers": [
        {"name": "a", "neural model": "relay", "rows": 3, "columns": 3},
        {"name": "b", "neural model": "izhikevich", "rows": 3, "columns": 3}]}],
        "connections": [{"name": "c", "from layer": "a", "to layer": "b",
                         "weight config": {"type": "flat", "weight": 0.5, "callback": "t_w",
                                           "delay callback": "t_d", "id": 1}}]}
    n = sg.Network(net)
    n.build_state()
    w = n.get_weight_matrix("c").to_np_array()
    assert np.array_equal(w, np.arange(81, dtype=np.float32) * 2)
    assert np.array_equal(n.get_weight_matrix("c", "delays").to_np_array(), np.arange(81) % 7)
    assert seen == {"w": 81, "d": 81}


def test_properties_and_json_roundtrip(sg, tmp_path):
    from tests.golden.cases import CASES
    net_dict = CASES["iz_opcodes"].net
    n = sg.Network(net_dict)
    path = str(tmp_path / "net.json")
    assert n.save(path)
    n2 = sg.Network(path)
    assert n2.obj
    n2.build_state()
    assert n2.get_weight_matrix("o_gap").size == 36 * 36
    p = sg.Properties({"a": "1", "b": True, "c": {"d": "x"}, "e": ["p", "q"], "f": [{"g": "h"}]})
    q = sg.Properties(p.obj).to_dict()
    assert q == {"a": "1", "b": "true", "c": {"d": "x"}, "e": ["p", "q"], "f": [{"g": "h"}]}


def test_state_save_load_roundtrip(sg, tmp_path):
    from tests.golden.cases import CASES
    net_dict = CASES["iz_plastic"].net
    n = sg.Network(net_dict)
    n.build_state()
    v = n.get_neuron_data("s", "e", "voltage").to_np_array()
    v[:] = np.linspace(-70, -50, v.size, dtype=np.float32)
    w = n.get_weight_matrix("p_ee").to_np_array()
    w[:] = np.random.default_rng(0).random(w.size).astype(np.float32)
    path = str(tmp_path / "state.bin")
    n.save_state(path)
    m = sg.Network(net_dict)
    m.build_state(path)
    assert np.array_equal(m.get_neuron_data("s", "e", "voltage").to_np_array(), v)
    assert np.array_equal(m.get_weight_matrix("p_ee").to_np_array(), w)


def test_randomized_divergent_overflow_is_refused(sg):
    """A randomized divergent projection whose flipped pairs give a
    destination more sources than the kernel has positions (where the
    reference writes past that destination's row) is refused at build."""
    net = {"structures": [{"name": "s", "layers": [
        {"name": "a", "neural model": "relay", "rows": 8, "columns": 8},
        {"name": "b", "neural model": "relay", "rows": 8, "columns": 8}]}],
        "connections": [{"name": "d", "from layer": "a", "to layer": "b", "type": "divergent",
                         "randomized projection": True, "plastic": False,
                         "arborized config": {"field size": 3, "stride": 1, "wrap": True},
                         "weight config": {"type": "flat", "weight": 1.0, "seed": 1}}]}
    n = sg.Network(net)
    n.build_state()
    assert not n.state
    assert "more than 9 sources" in sg.last_error()
