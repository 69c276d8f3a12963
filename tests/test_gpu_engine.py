"""GPU tests of the engine paths: the fused game_of_life step with ping-pong
history buffers, CUDA-graph replay across calls of uneven length, and the full
2048x2048 configuration, all bit-exact against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    from synaptogenesis_gb300 import syngen
    assert syngen.get_gpus(), "no CUDA GPU visible"
    syngen.set_warnings(False)
    return syngen


def gol_net(rows, cols, field=3, wrap=True, delay=0, weight=1.0, diagonal=False, **rule):
    return {"structures": [{"name": "g", "type": "parallel", "layers": [
        dict({"name": "board", "neural model": "game_of_life", "rows": rows, "columns": cols},
             **rule)]}],
        "connections": [{"name": "nbr", "from layer": "board", "to layer": "board",
                         "type": "convergent", "convolutional": True, "plastic": False,
                         "opcode": "add", "delay": delay,
                         "weight config": {"type": "flat", "weight": weight, "diagonal": diagonal},
                         "arborized config": {"field size": field, "wrap": wrap}}]}


@pytest.mark.parametrize("variant", [
    dict(wrap=False), dict(delay=5), dict(diagonal=True, survival_min=3, survival_max=4),
    dict(weight=2.0, survival_min=4, survival_max=6, birth_min=6, birth_max=6),
    dict(wrap=False, delay=31, birth_min=2, birth_max=3)])
def test_gol_kernel_variants_match_oracle(sg, variant):
    """Bit-sliced path (0/1 weights) and its fallback (other weights)."""
    rows, cols = 37, 128
    words = np.random.default_rng(7).integers(0, 2**32, rows * cols, dtype=np.uint64).astype(np.uint32)
    go, gi, oo, oi = run_both(sg, gol_net(rows, cols, **variant), words, [19, 22])
    assert np.array_equal(go, oo)
    assert np.array_equal(gi, oi)


def run_both(sg, net_dict, words, chunks, graphs=True):
    from oracle.oracle import OracleNetwork
    net = sg.Network(net_dict)
    net.build_state()
    net.get_neuron_data("g", "board", "output").to_np_array().view(np.uint32)[:] = words
    with sg.Engine(net, None, {"graphs": graphs, "graph steps": 8}) as eng:
        for n in chunks:
            assert eng.step(n) == n
    got_out = net.get_neuron_data("g", "board", "output").to_np_array().view(np.uint32).copy()
    got_in = net.get_neuron_data("g", "board", "input").to_np_array().copy()
    onet = OracleNetwork(net_dict)
    onet.get_neuron_data("board", "output")[:] = words
    for _ in range(sum(chunks)):
        onet.step()
    return got_out, got_in, onet.get_neuron_data("board", "output"), onet.get_neuron_data("board", "input")


@pytest.mark.parametrize("graphs", [True, False])
def test_fused_gol_matches_oracle_across_uneven_chunks(sg, graphs):
    rows, cols = 96, 160
    words = np.random.default_rng(5).integers(0, 2**32, rows * cols, dtype=np.uint64).astype(np.uint32)
    go, gi, oo, oi = run_both(sg, gol_net(rows, cols, survival_min=2, survival_max=4,
                                          birth_min=3, birth_max=3), words, [37, 9, 20, 1])
    assert np.array_equal(go, oo)
    assert np.array_equal(gi, oi)


def test_fused_gol_field5_matches_oracle(sg):
    rows, cols = 40, 72
    words = np.random.default_rng(6).integers(0, 2**32, rows * cols, dtype=np.uint64).astype(np.uint32)
    go, gi, oo, oi = run_both(sg, gol_net(rows, cols, field=5, survival_min=4, survival_max=9,
                                          birth_min=5, birth_max=7), words, [25, 14])
    assert np.array_equal(go, oo)
    assert np.array_equal(gi, oi)


def test_gol_2048_full_size_matches_oracle(sg):
    side = 2048
    rng = np.random.default_rng(1)
    words = (rng.random(side * side) < 0.3).astype(np.uint32) << np.uint32(31)
    go, gi, oo, oi = run_both(sg, gol_net(side, side), words, [12, 7])
    assert np.array_equal(go, oo)
    assert np.array_equal(gi, oi)


def test_izhikevich_graph_replay_equals_stepwise(sg):
    """Same network advanced with captured graphs and with plain launches."""
    import copy
    from tests.golden.cases import CASES
    net_dict = copy.deepcopy(CASES["iz_c0_32"].net)
    net_dict["structures"][0]["layers"][0]["init config"] = {"type": "flat", "value": 0.4}
    results = []
    for graphs in (True, False):
        net = sg.Network(net_dict)
        net.build_state()
        n = net.get_weight_matrix("c_rec", "weights").size
        net.get_weight_matrix("c_rec", "weights").to_np_array()[:] = \
            np.random.default_rng(3).uniform(0, 0.2, n).astype(np.float32)
        net.get_weight_matrix("c_in", "short term w").to_np_array()[:] = 0.5
        net.get_neuron_data("s", "iz", "input")
        with sg.Engine(net, None, {"graphs": graphs, "graph steps": 6}) as eng:
            eng.step(29)
            eng.step(31)
        results.append({k: net.get_neuron_data("s", "iz", k).to_np_array().copy()
                        for k in ("voltage", "recovery", "output", "nmda", "time since spike")})
    for k in results[0]:
        assert np.array_equal(results[0][k].view(np.uint32), results[1][k].view(np.uint32)), k


@pytest.mark.parametrize("rows,cols,rule", [
    (96, 160, dict(survival_min=2, survival_max=3, birth_min=3, birth_max=3)),
    (20, 32, dict(survival_min=2, survival_max=4, birth_min=3, birth_max=3)),
    (130, 288, dict(diagonal=True, survival_min=3, survival_max=4, birth_min=3, birth_max=5)),
    (257, 64, dict(survival_min=1, survival_max=5, birth_min=2, birth_max=3)),
    # boards 1024, 2048 and 4096 cells wide take the full-width strip kernel
    (40, 1024, dict(survival_min=2, survival_max=3, birth_min=3, birth_max=3)),
    (70, 2048, dict(diagonal=True, survival_min=3, survival_max=4, birth_min=3, birth_max=5)),
    (17, 2048, dict(survival_min=1, survival_max=5, birth_min=2, birth_max=3)),
    (33, 4096, dict(survival_min=2, survival_max=3, birth_min=3, birth_max=3)),
    (24, 4096, dict(diagonal=True, survival_min=2, survival_max=6, birth_min=4, birth_max=4))])
def test_gol_whole_runs_equal_per_step_path(sg, rows, cols, rule):
    """Without an environment a toroidal game_of_life board advances whole runs
    on bit planes (many steps per launch); words and the input register equal
    the per-step path's and the oracle's for step counts around the launch
    size (16 steps)."""
    words = np.random.default_rng(rows * cols).integers(0, 2**32, rows * cols,
                                                       dtype=np.uint64).astype(np.uint32)
    chunks = [1, 16, 17, 33, 100, 5]
    net_dict = gol_net(rows, cols, **rule)
    results = []
    for whole in (True, False):
        net = sg.Network(net_dict)
        net.build_state()
        net.get_neuron_data("g", "board", "output").to_np_array().view(np.uint32)[:] = words
        with sg.Engine(net, None, {"whole runs": whole}) as eng:
            for n in chunks:
                assert eng.step(n) == n
                results.append((whole, n,
                                net.get_neuron_data("g", "board", "output").to_np_array()
                                .view(np.uint32).copy(),
                                net.get_neuron_data("g", "board", "input").to_np_array().copy()))
    half = len(results) // 2
    for (_, n, wa, ia), (_, _, wb, ib) in zip(results[:half], results[half:]):
        assert np.array_equal(wa, wb), n
        assert np.array_equal(ia, ib), n
    go, gi, oo, oi = run_both(sg, net_dict, words, chunks)
    assert np.array_equal(go, oo)
    assert np.array_equal(gi, oi)
