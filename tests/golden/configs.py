"""The measured configurations at their stated sizes, seeded, for the parity
tests at size, the fixtures recorded from the reference and the benchmark.

* ``c0``: a 32x32 relay layer driven by Poisson spikes (probability 0.01 per
  1 ms step, value 1.0) feeds a 32x32 Izhikevich regular-spiking layer through
  a 5x5 wrapping convergent excitatory connection (weights U(0, 0.5)); an
  inhibitory recurrent fully connected connection at 20% density (weights
  U(0, 0.2)); delays U{0..3}; v0 = -65, u0 = b v0; no plasticity.
* ``c1``: game_of_life on a 2048x2048 toroidal board, 3x3 neighbourhood
  without the centre, B3/S23, cells alive with probability 0.3 (seed 1).
* ``c2``: three 256x256 Izhikevich layers (80% regular / 20% fast spiking,
  drawn per neuron by seed 2), L1->L2 convergent 9x9 wrapping with STDP
  (learning rate 0.004, weights U(0, 0.3)), L2->L3 divergent 3x3 stride 2
  (U(0, 0.3)), L3->L1 one-to-one inhibitory (0.5), and a fully connected
  4096x4096 projection between the central 64x64 windows of L2 and L3
  (subset connection, weights max(0, N(0, 0.05))); delays U{0..3}; a 5 Hz
  Poisson drive of value 20 into L1's input current.

Every random quantity is injected, since the reference's own initialisers
draw from unseeded generators.  Records are kept as digests: a 64-bit
BLAKE2b of each step's output words per layer, plus the per-step spike count
(bit 31 of the newest word), so fixtures stay small at these sizes.
"""
import hashlib

import numpy as np

from tests.golden.cases import Case

C2_SIDE = 256
C2_SUBSET = (96, 160)          # rows / columns of the 64x64 windows of L2 and L3
C2_DRIVE_P = 0.005             # 5 Hz at 1 ms per step
C2_DRIVE_VALUE = 20.0


def digest(arr):
    """64-bit BLAKE2b digest of an array's bytes, as an unsigned integer."""
    a = np.ascontiguousarray(arr)
    return np.uint64(int.from_bytes(hashlib.blake2b(a.tobytes(), digest_size=8).digest(), "little"))


def spike_count(words):
    """Neurons whose newest output bit (bit 31 of history word 0) is set."""
    return int(np.count_nonzero(np.asarray(words).view(np.uint32) >> np.uint32(31)))


def _layer(name, model, rows, cols, **kw):
    d = {"name": name, "neural model": model, "rows": rows, "columns": cols}
    d.update(kw)
    return d


# ---------------------------------------------------------------------------
# C0: plain 32x32 Izhikevich
# ---------------------------------------------------------------------------
def c0_net(side=32):
    return {"structures": [{"name": "s", "type": "parallel", "layers": [
        _layer("in", "relay", side, side),
        _layer("iz", "izhikevich", side, side, params="regular")]}],
        "connections": [
            {"name": "c_in", "from layer": "in", "to layer": "iz", "type": "convergent",
             "plastic": False, "opcode": "add",
             "arborized config": {"field size": 5, "wrap": True}},
            {"name": "c_rec", "from layer": "iz", "to layer": "iz",
             "type": "fully connected", "plastic": False, "opcode": "sub"}]}


def c0_inject(rng, sizes, side=32):
    n = side * side
    nin, nrec = sizes["conn:c_in"], sizes["conn:c_rec"]
    v0 = np.full(n, -65.0, np.float32)
    return {("matrix", "c_in", "weights"): rng.uniform(0, 0.5, nin).astype(np.float32),
            ("matrix", "c_in", "short term w"): np.full(nin, 0.5, np.float32),
            ("matrix", "c_in", "delays"): rng.integers(0, 4, nin).astype(np.int32),
            ("matrix", "c_rec", "weights"):
                (rng.uniform(0, 0.2, nrec) * (rng.random(nrec) < 0.2)).astype(np.float32),
            ("matrix", "c_rec", "delays"): rng.integers(0, 4, nrec).astype(np.int32),
            ("neuron", "s", "iz", "voltage"): v0,
            ("neuron", "s", "iz", "recovery"): (np.float32(0.2) * v0).astype(np.float32)}


def c0_case(steps=1000):
    return Case("c0_1000", c0_net(), steps, 201, inject=c0_inject,
                inputs={"in": lambda rng, t, m: (rng.random(m) < 0.01) * 1.0},
                record=[("s", "iz"), ("s", "in")],
                final=[("neuron", "s", "iz", k) for k in
                       ("voltage", "recovery", "post trace", "time since spike", "output")]
                + [("matrix", c, k) for c in ("c_in", "c_rec")
                   for k in ("short trace", "long trace", "time since spike")],
                learning=False)


# ---------------------------------------------------------------------------
# C1: game_of_life 2048x2048
# ---------------------------------------------------------------------------
def c1_net(side=2048):
    return {"structures": [{"name": "g", "type": "parallel", "layers": [
        _layer("board", "game_of_life", side, side, survival_min=2, survival_max=3,
               birth_min=3, birth_max=3)]}],
        "connections": [{"name": "nbr", "from layer": "board", "to layer": "board",
                         "type": "convergent", "convolutional": True, "plastic": False,
                         "opcode": "add",
                         "weight config": {"type": "flat", "weight": 1.0, "diagonal": False},
                         "arborized config": {"field size": 3, "wrap": True}}]}


def c1_initial_words(side=2048, seed=1, p=0.3):
    rng = np.random.default_rng(seed)
    return (rng.random(side * side) < p).astype(np.uint32) << np.uint32(31)


# ---------------------------------------------------------------------------
# C2: three 256x256 Izhikevich layers with STDP and a 4096x4096 projection
# ---------------------------------------------------------------------------
def c2_net(side=C2_SIDE, device_drive=None):
    """The network; ``device_drive`` (a seed) replaces the callback drive of
    L1 by the on-device Poisson init config of the same rate and value."""
    def layer(name, drive=False):
        d = _layer(name, "izhikevich", side, side, params="regular")
        if drive and device_drive is not None:
            d["init config"] = {"type": "poisson", "rate": 5, "value": C2_DRIVE_VALUE,
                                "seed": device_drive}
        return d
    lo, hi = C2_SUBSET
    return {"structures": [{"name": "s", "type": "parallel", "layers": [
        layer("L1", drive=True), layer("L2"), layer("L3")]}],
        "connections": [
            {"name": "c12", "from layer": "L1", "to layer": "L2", "type": "convergent",
             "opcode": "add", "plastic": True, "learning rate": 0.004,
             "arborized config": {"field size": 9, "wrap": True}},
            {"name": "c23", "from layer": "L2", "to layer": "L3", "type": "divergent",
             "opcode": "add", "plastic": False,
             "arborized config": {"field size": 3, "stride": 2}},
            {"name": "c31", "from layer": "L3", "to layer": "L1", "type": "one to one",
             "opcode": "sub", "plastic": False},
            {"name": "c23s", "from layer": "L2", "to layer": "L3", "type": "subset",
             "opcode": "add", "plastic": False,
             "subset config": {"from row start": lo, "from row end": hi, "from column start": lo,
                               "from column end": hi, "to row start": lo, "to row end": hi,
                               "to column start": lo, "to column end": hi}}]}


def c2_inject(rng, sizes, side=C2_SIDE):
    n = side * side
    d = {}
    prng = np.random.default_rng(2)
    for lname in ("L1", "L2", "L3"):
        fast = prng.random(n) < 0.2           # 80% regular, 20% fast spiking
        vals = {"a": np.where(fast, 0.1, 0.02), "b": np.full(n, 0.2),
                "c": np.full(n, -65.0), "d": np.where(fast, 2.0, 8.0),
                "voltage": np.full(n, -65.0)}
        for k, v in vals.items():
            d[("neuron", "s", lname, k)] = v.astype(np.float32)
        d[("neuron", "s", lname, "recovery")] = np.full(n, np.float32(0.2) * np.float32(-65.0),
                                                        np.float32)
    for c in ("c12", "c23", "c31", "c23s"):
        m = sizes["conn:" + c]
        if c == "c31":
            w = np.full(m, 0.5, np.float32)
        elif c == "c23s":
            w = np.maximum(0.0, rng.normal(0.0, 0.05, m)).astype(np.float32)
        else:
            w = rng.uniform(0.0, 0.3, m).astype(np.float32)
        d[("matrix", c, "weights")] = w
        d[("matrix", c, "delays")] = rng.integers(0, 4, m).astype(np.int32)
        if c != "c23s":
            # "short term w" of convergent / divergent / one-to-one matrices
            # starts at 0 in the reference (it compares the connection type with
            # opcodes); they get the "add" value U = 0.5
            d[("matrix", c, "short term w")] = np.full(m, 0.5, np.float32)
    return d


def c2_drive(rng, t, m):
    return (rng.random(m) < C2_DRIVE_P) * C2_DRIVE_VALUE


C2_FINAL_NEURON = ("voltage", "recovery", "post trace", "time since spike", "output")
C2_FINAL_MATRIX = {"c12": ("weights", "weight derivatives", "presyn trace", "short term R",
                           "short term w", "short trace", "long trace", "time since spike"),
                   "c23s": ("short trace", "long trace", "time since spike")}


def c2_case(steps=1000):
    final = [("neuron", "s", l, k) for l in ("L1", "L2", "L3") for k in C2_FINAL_NEURON]
    final += [("matrix", c, k) for c, ks in C2_FINAL_MATRIX.items() for k in ks]
    return Case("c2_1000", c2_net(), steps, 221, inject=c2_inject, inputs={"L1": c2_drive},
                record=[("s", "L1"), ("s", "L2"), ("s", "L3")], final=final, learning=True)


# Split points of the C2 and C0 runs at which full state digests are taken
# (the first 100 steps must match bit for bit; rates over the whole run).
CHECKPOINTS = (100,)
