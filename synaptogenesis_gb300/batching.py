"""Host-side helpers of the batched Izhikevich runner.

* ``counter_uniform`` / ``counter_below``: numpy restatement of the
  counter-based generator in csrc/counter_rng.h (SplitMix64 finaliser), so the
  host can rebuild any generated weight, delay or input exactly.
* ``batch_instances``: the seeded batch of uneven instances (sides uniform in
  16..128, Izhikevich a/b/c/d within +-10% of regular spiking, one seed each).
* ``plain_network``: one instance as an ordinary network in the reference's
  JSON schema plus its injected state and per-step inputs, for the
  layer-by-layer path -- whose spike raster must equal the batch's.
* ``shard_instances``: partition of instances over ranks (independent
  instances, no exchange between ranks), largest first onto the least loaded.
"""
import numpy as np

RNG_CONV_WEIGHT, RNG_FC_WEIGHT, RNG_FC_MASK, RNG_FC_DELAY, RNG_INPUT = 1, 2, 3, 4, 5
_M = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix(z):
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def counter_bits(seed, stream, index):
    index = np.asarray(index, dtype=np.uint64)
    with np.errstate(over="ignore"):
        base = (np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15)
                + np.uint64(stream) * np.uint64(0xD1B54A32D192ED03))
        return _mix(base + index)


def counter_uniform(seed, stream, index):
    """float32 in [0, 1) with 24 random bits (rng_uniform)."""
    b = counter_bits(seed, stream, index) >> np.uint64(40)
    return b.astype(np.float32) * np.float32(1.0 / 16777216.0)


def counter_below(seed, stream, index, n):
    """Integer in [0, n) (rng_below)."""
    return ((counter_bits(seed, stream, index) >> np.uint64(32)) % np.uint64(n)).astype(np.int32)


REGULAR = dict(a=0.02, b=0.2, c=-65.0, d=8.0)


def instance(side, seed, a=0.02, b=0.2, c=-65.0, d=8.0, rows=None, cols=None):
    """One instance of the plain Izhikevich configuration: relay drive 10 Hz at
    1 ms steps (value 1.0 with probability 0.01), convergent 5x5 wrapping
    excitatory weights U(0, 0.5) with short term w 0.5, recurrent inhibitory
    weights U(0, 0.2) at 20% density, delays U{0..3}, v0 = -65."""
    return dict(rows=int(rows or side), cols=int(cols or side), a=float(a), b=float(b),
                c=float(c), d=float(d), v0=-65.0, seed=int(seed), input_rate=0.01,
                input_value=1.0, conv_field=5, conv_wmax=0.5, conv_stp_w=0.5,
                conv_conductance=1.0, fc_wmax=0.2, fc_density=0.2, fc_stp_w=0.5,
                fc_conductance=1.0, fc_max_delay=3)


def batch_instances(count=256, seed=3, smin=16, smax=128):
    """``count`` instances with sides uniform in [smin, smax] and a, b, c, d
    each scaled by U(0.9, 1.1) around regular spiking, seeded by ``seed``."""
    rng = np.random.default_rng(seed)
    sides = rng.integers(smin, smax + 1, count)
    scale = rng.uniform(0.9, 1.1, (count, 4))
    out = []
    for i in range(count):
        p = {k: float(np.float32(REGULAR[k] * scale[i, j])) for j, k in enumerate("abcd")}
        out.append(instance(int(sides[i]), seed * 100003 + i, **p))
    return out


def fc_dense(inst):
    """Recurrent weights and delays in the reference's CPU layout [to][from]."""
    n = inst["rows"] * inst["cols"]
    idx = np.arange(n * n, dtype=np.uint64)
    mask = counter_uniform(inst["seed"], RNG_FC_MASK, idx) < np.float32(inst["fc_density"])
    w = counter_uniform(inst["seed"], RNG_FC_WEIGHT, idx) * np.float32(inst["fc_wmax"])
    w = np.where(mask, w, np.float32(0.0)).astype(np.float32)
    delays = counter_below(inst["seed"], RNG_FC_DELAY, idx, inst["fc_max_delay"] + 1)
    return w, delays


def conv_dense(inst):
    """Convergent weights in the CPU layout [to][k]."""
    n = inst["rows"] * inst["cols"]
    K = inst["conv_field"] ** 2
    idx = np.arange(n * K, dtype=np.uint64)
    return counter_uniform(inst["seed"], RNG_CONV_WEIGHT, idx) * np.float32(inst["conv_wmax"])


def relay_input(inst, step):
    """Relay layer input of ``step``."""
    n = inst["rows"] * inst["cols"]
    idx = np.uint64(step) * np.uint64(n) + np.arange(n, dtype=np.uint64)
    u = counter_uniform(inst["seed"], RNG_INPUT, idx)
    return np.where(u < np.float32(inst["input_rate"]), np.float32(inst["input_value"]),
                    np.float32(0.0)).astype(np.float32)


def plain_network(inst):
    """(network dict, injections, input function) of one instance for the
    layer-by-layer path.  Injections are keyed like the parity harness:
    ("matrix", connection, key) / ("neuron", structure, layer, key)."""
    rows, cols = inst["rows"], inst["cols"]
    n = rows * cols
    layer = lambda name, model, **kw: dict({"name": name, "neural model": model, "rows": rows,
                                            "columns": cols}, **kw)
    net = {"structures": [{"name": "s", "type": "parallel", "layers": [
        layer("in", "relay"), layer("iz", "izhikevich", params="regular")]}],
        "connections": [
            {"name": "c_in", "from layer": "in", "to layer": "iz", "type": "convergent",
             "plastic": False, "opcode": "add",
             "conductance": str(inst["conv_conductance"]),
             "arborized config": {"field size": inst["conv_field"], "wrap": True}},
            {"name": "c_rec", "from layer": "iz", "to layer": "iz", "type": "fully connected",
             "plastic": False, "opcode": "sub", "myelinated": True,
             "conductance": str(inst["fc_conductance"])}]}
    w, delays = fc_dense(inst)
    cw = conv_dense(inst)
    v0 = np.full(n, inst["v0"], np.float32)
    inj = {("matrix", "c_in", "weights"): cw,
           ("matrix", "c_in", "short term w"): np.full(cw.size, inst["conv_stp_w"], np.float32),
           ("matrix", "c_rec", "weights"): w,
           ("matrix", "c_rec", "short term w"): np.full(w.size, inst["fc_stp_w"], np.float32),
           ("matrix", "c_rec", "delays"): delays,
           ("neuron", "s", "iz", "voltage"): v0,
           ("neuron", "s", "iz", "recovery"): (np.float32(inst["b"]) * v0).astype(np.float32)}
    for k in "abcd":
        inj[("neuron", "s", "iz", k)] = np.full(n, inst[k], np.float32)
    return net, inj, (lambda step: relay_input(inst, step))


def instance_cost(inst):
    """Relative per-step work of an instance: its recurrent synapses."""
    n = inst["rows"] * inst["cols"]
    return n * n * inst["fc_density"] + n * inst["conv_field"] ** 2


def shard_instances(instances, rank, world):
    """Indices of the instances rank ``rank`` of ``world`` runs: largest first,
    each onto the currently least loaded rank (ties to the lowest rank)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside a world of %d" % (rank, world))
    order = sorted(range(len(instances)), key=lambda i: (-instance_cost(instances[i]), i))
    load = [0.0] * world
    owner = {}
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += instance_cost(instances[i])
    return [i for i in range(len(instances)) if owner[i] == rank]
