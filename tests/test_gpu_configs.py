"""GPU parity at the measured configurations' stated sizes and lengths,
against digests recorded from the reference's own CPU library
(tests/golden/make_golden.py, one OpenMP thread for the plastic network):

* c0: the 32x32 Izhikevich network for 1000 steps.  The first 100 steps'
  output words and the state after step 100 are bit-exact; the firing rate
  over 1000 steps is within 1%; and (a stronger claim than the rate) every
  step's words and the final state are bit-exact too.
* c2: three 256x256 Izhikevich layers with STDP on the 9x9 convergent
  connection, the divergent stride-2 and one-to-one connections and the
  4096x4096 subset connection, for 1000 steps: the same checks per layer.
* c1: game_of_life on 2048x2048 for 10,000 steps: the words and the input
  register after every 1000 steps are bit-exact.
* c3: the three largest instances of the 256-instance batch equal the same
  instances run by the layer-by-layer path for 64 steps.
"""
import numpy as np
import pytest

from tests.golden import configs
from tests.harness import load_fixture, run_digest, run_gol_digest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    from synaptogenesis_gb300 import syngen
    assert syngen.get_gpus(), "no CUDA GPU visible"
    syngen.set_warnings(False)
    return syngen


def _check_digests(got, want, bit_layers):
    first = 100
    for k, w in want.items():
        if k.startswith("digest/"):
            g = got[k]
            assert g.shape == w.shape, k
            bad = np.flatnonzero(g[:first] != w[:first])
            assert bad.size == 0, "%s: first %d steps differ from step %d" % (k, first, bad[0])
        elif k.startswith("final@%d/" % first):
            assert got[k][0] == w[0], k
    for layer in bit_layers:
        g = int(got["count/" + layer].sum())
        w = int(want["count/" + layer].sum())
        assert w > 0, "no spikes in %s: the rate check would be vacuous" % layer
        assert abs(g - w) <= 0.01 * w, (layer, g, w)
    # every step and the final state, bit for bit
    for k, w in want.items():
        if k.startswith("digest/") or k.startswith("count/"):
            bad = np.flatnonzero(got[k] != w)
            assert bad.size == 0, "%s differs from step %d" % (k, bad[0])
        elif k.startswith("final@"):
            assert got[k][0] == w[0], k


def test_c0_izhikevich_1000_steps(sg):
    case = configs.c0_case()
    got = run_digest(case, sg, checkpoints=configs.CHECKPOINTS)
    _check_digests(got, load_fixture(case.name), ["s/iz"])


def test_c2_plastic_izhikevich_1000_steps(sg):
    case = configs.c2_case()
    got = run_digest(case, sg, checkpoints=configs.CHECKPOINTS)
    _check_digests(got, load_fixture(case.name), ["s/L1", "s/L2", "s/L3"])


def test_c1_game_of_life_10000_steps(sg):
    got = run_gol_digest(sg, 2048, 10000, 1000)
    want = load_fixture("c1_10000")
    for k in ("digest/words", "digest/input"):
        bad = np.flatnonzero(got[k] != want[k])
        assert bad.size == 0, "%s differs after %d steps" % (k, 1000 * (bad[0] + 1))


def test_c3_largest_instances_match_plain_path(sg):
    """The full 256-instance batch, stepped 64 times: the three largest
    instances' output words (every 32 steps), voltages and recoveries equal
    those of the layer-by-layer path."""
    from synaptogenesis_gb300 import batching
    from tests.test_gpu_batch import as_case
    from tests.harness import run_library
    insts = batching.batch_instances(256, 3)
    largest = sorted(range(len(insts)), key=lambda i: (-insts[i]["rows"] * insts[i]["cols"], i))[:3]
    assert all(insts[i]["rows"] >= 120 for i in largest)
    words = {i: [] for i in largest}
    with sg.Batch(insts) as b:
        for _ in range(2):
            b.step(32)
            for i in largest:
                words[i].append(b.read(i, "output"))
        finals = {i: (b.read(i, "voltage").view(np.uint32), b.read(i, "recovery").view(np.uint32))
                  for i in largest}
    for i in largest:
        want = run_library(as_case(insts[i], 64), sg, 64)
        rec = want["rec/s/iz"]
        assert np.array_equal(words[i][0], rec[31]), i
        assert np.array_equal(words[i][1], rec[63]), i
        assert np.array_equal(finals[i][0], want["neuron/s/iz/voltage"]), i
        assert np.array_equal(finals[i][1], want["neuron/s/iz/recovery"]), i
