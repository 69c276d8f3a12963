"""GPU tests of the batched Izhikevich runner: every instance's spike raster,
voltages and recoveries equal, bit for bit, those of the same instance built as
an ordinary network and run by the layer-by-layer path (itself pinned to the
reference by the golden fixtures), and of the CPU oracle for a small instance.
Tile shapes, CUDA-graph replay and uneven step counts do not change results."""
import numpy as np
import pytest

from tests.golden.cases import Case
from tests.harness import run_library, run_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    from synaptogenesis_gb300 import syngen
    assert syngen.get_gpus(), "no CUDA GPU visible"
    syngen.set_warnings(False)
    return syngen


def as_case(inst, steps):
    from synaptogenesis_gb300.batching import plain_network, relay_input
    net, inj, _ = plain_network(inst)
    return Case("batch_%d" % inst["seed"], net, steps, 0, inject=lambda rng, sizes: dict(inj),
                inputs={"in": lambda rng, t, m: relay_input(inst, t)},
                record=[("s", "iz")],
                final=[("neuron", "s", "iz", "voltage"), ("neuron", "s", "iz", "recovery")])


def mixed_instances(sides, seed=11):
    from synaptogenesis_gb300 import batching
    rng = np.random.default_rng(seed)
    out = []
    for i, s in enumerate(sides):
        sc = rng.uniform(0.9, 1.1, 4)
        p = {k: float(np.float32(batching.REGULAR[k] * sc[j])) for j, k in enumerate("abcd")}
        inst = batching.instance(s, 1000 * seed + i, **p)
        inst["input_rate"] = 0.05          # more activity for a short run
        out.append(inst)
    return out


def run_batch(sg, insts, chunks, tile=None):
    """Steps a batch in ``chunks`` and returns, per instance, the output word
    after every 32nd step (each word holds the last 32 steps' spikes) and the
    final voltage and recovery."""
    words = [[] for _ in insts]
    with sg.Batch(insts, tile=tile) as b:
        done = 0
        for n in chunks:
            b.step(n)
            done += n
            if done % 32 == 0:
                for i in range(len(insts)):
                    words[i].append(b.read(i, "output"))
        finals = [(b.read(i, "voltage").view(np.uint32), b.read(i, "recovery").view(np.uint32))
                  for i in range(len(insts))]
        rep = b.report()
    return words, finals, rep


def test_batch_matches_plain_path(sg):
    insts = mixed_instances([16, 19, 23, 30, 37, 45, 33, 20])
    steps = 64
    words, finals, rep = run_batch(sg, insts, [32, 32])
    assert int(rep.properties["kernel launches"]) == steps
    assert all(len(w) == 2 for w in words)
    spikes = 0
    for i, inst in enumerate(insts):
        want = run_library(as_case(inst, steps), sg, steps)
        rec = want["rec/s/iz"]
        for j, w in enumerate(words[i]):
            assert np.array_equal(w, rec[32 * j + 31]), (i, j)
        assert np.array_equal(finals[i][0], want["neuron/s/iz/voltage"]), i
        assert np.array_equal(finals[i][1], want["neuron/s/iz/recovery"]), i
        spikes += int(np.unpackbits(rec[31::32].view(np.uint8)).sum())
    assert spikes > 0, "no activity: the comparison would be vacuous"


def test_batch_matches_oracle(sg):
    inst = mixed_instances([12], seed=5)[0]
    steps = 64
    words, finals, _ = run_batch(sg, [inst], [32, 32], tile=(2, 1))
    want = run_oracle(as_case(inst, steps), steps)
    assert np.array_equal(words[0][0], want["rec/s/iz"][31])
    assert np.array_equal(words[0][1], want["rec/s/iz"][63])
    assert np.array_equal(finals[0][0], want["neuron/s/iz/voltage"])
    assert np.array_equal(finals[0][1], want["neuron/s/iz/recovery"])


@pytest.mark.parametrize("tile", [(1, 1), (8, 1), (2, 4), (4, 2)])
def test_batch_tiles_and_graphs_agree(sg, tile):
    """Every tile shape and any split of the steps (graph replays of 32 plus
    single launches) give the autotuned batch's results."""
    insts = mixed_instances([16, 70, 24, 96, 41, 17, 64, 33, 128], seed=7)
    ref_words, ref_finals, rep = run_batch(sg, insts, [32, 64])
    assert len(rep.child_arrays["autotune"]) >= 2
    words, finals, _ = run_batch(sg, insts, [5, 27, 33, 31], tile=tile)
    for i in range(len(insts)):
        assert len(words[i]) == len(ref_words[i]) == 2
        for a, b in zip(words[i], ref_words[i]):
            assert np.array_equal(a, b), (tile, i)
        assert np.array_equal(finals[i][0], ref_finals[i][0]), (tile, i)
        assert np.array_equal(finals[i][1], ref_finals[i][1]), (tile, i)


def test_batch_full_configuration_smoke(sg):
    """The 256-instance configuration builds, autotunes and steps; its synapse
    count equals the sum of the instances' non-zero recurrent weights."""
    from synaptogenesis_gb300 import batching
    insts = batching.batch_instances(256, 3)
    with sg.Batch(insts) as b:
        b.step(40)
        rep = b.report().properties
        v = b.read(255, "voltage")
    assert int(rep["instances"]) == 256
    assert int(rep["kernel launches"]) == 40
    assert np.isfinite(v).all()
    # exact count for a few instances, from the host restatement
    small = [i for i, x in enumerate(insts) if x["rows"] <= 24][:3]
    with sg.Batch([insts[i] for i in small]) as b:
        nz = int(b.report().properties["fc synapses"])
    want = sum(int((batching.fc_dense(insts[i])[0] != 0).sum()) for i in small)
    assert nz == want
