"""Runs golden cases on the oracle or on the GB300 library and compares results."""
import os

import numpy as np

from tests.golden.cases import CASES

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_fixture(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def case_sizes(case):
    """Layer sizes and weight counts per connection.  Sizes do not depend on
    delays, so connections are built myelinated here: distance delays of large
    layers exceed a BIT history word, and cases inject their delays anyway."""
    import copy
    from oracle.oracle import OracleNetwork
    net = copy.deepcopy(case.net)
    for c in net["connections"]:
        c["myelinated"] = True
    onet = OracleNetwork(net)
    sizes = {l.name: l.size for l in onet.layers}
    sizes.update({"conn:" + c.name: c.num_weights for c in onet.conns})
    sizes.update({"dense:" + c.name: c.dense_num_weights for c in onet.conns})
    return sizes


def _as_u32(a):
    a = np.asarray(a)
    return a.view(np.uint32) if a.dtype == np.float32 else a


def _oracle_network(case):
    """The case's network on the CPU oracle with every injection applied."""
    from oracle.oracle import OracleNetwork
    from tests.golden.cases import callback_injections
    sizes = case_sizes(case)
    injections = case.injections(sizes)
    # dense weights of sparse connections through the weight callback; the
    # other injections go into the built state
    _, _, weight_arrays, _ = callback_injections(case.net, injections)
    net_dict, _, _, _ = callback_injections(
        case.net, {k: v for k, v in injections.items() if k[2] == "init weights"})
    for c in net_dict["connections"]:
        # injected delays replace the distance delays, which large layers
        # could not hold in one BIT history word
        if ("matrix", c["name"], "delays") in injections:
            c["myelinated"] = True
    net = OracleNetwork(net_dict, weight_callbacks={
        "golden_weight": lambda ID, w: w.__setitem__(slice(None), weight_arrays[ID])})
    for key, arr in injections.items():
        if key[2] == "init weights":
            continue
        if key[0] == "neuron":
            dst = net.get_neuron_data(key[2], key[3])
        else:
            dst = net.get_weight_matrix(key[1], key[2])
        assert dst.size == arr.size, key
        dst.view(arr.dtype)[:] = arr
    return net, sizes


def _final_key(key):
    return ("neuron/%s/%s/%s" if key[0] == "neuron" else "matrix/%s/%s") % tuple(key[1:])


def _oracle_final(net, key):
    if key[0] == "neuron":
        return _as_u32(net.get_neuron_data(key[2], key[3]).copy())
    return _as_u32(net.get_weight_matrix(key[1], key[2]).copy())


def run_oracle(case, steps=None):
    """Runs ``case`` on the CPU oracle; returns the fixture-shaped dict."""
    steps = case.steps if steps is None else steps
    net, sizes = _oracle_network(case)
    inputs = case.input_arrays(sizes, steps)
    rec = {k: [] for k in case.record}
    for t in range(steps):
        net.step(inputs[t], learning=case.learning)
        for (s, l) in case.record:
            rec[(s, l)].append(net.get_neuron_data(l, "output")[:sizes[l]].copy())
    out = {"rec/%s/%s" % k: np.stack(v) for k, v in rec.items()}
    for key in case.final:
        out[_final_key(key)] = _oracle_final(net, key)
    return out


def run_oracle_digest(case, steps, checkpoints=()):
    """``run_digest`` on the CPU oracle: per-step output digests and spike
    counts, state digests at the checkpoints within ``steps`` and at the end."""
    from tests.golden.cases import _rng
    from tests.golden.configs import digest, spike_count
    net, sizes = _oracle_network(case)
    rng = _rng(case.seed + 1000)
    dig = {k: [] for k in case.record}
    cnt = {k: [] for k in case.record}
    out = {}
    marks = set(c for c in checkpoints if 0 < c < steps) | {steps}
    for t in range(steps):
        inputs = {name: fn(rng, t, sizes[name]).astype(np.float32)
                  for name, fn in sorted(case.inputs.items())}
        net.step(inputs, learning=case.learning)
        for (s, l) in case.record:
            words = net.get_neuron_data(l, "output")[:sizes[l]]
            dig[(s, l)].append(digest(words))
            cnt[(s, l)].append(spike_count(words))
        if t + 1 in marks:
            for key in case.final:
                out["final@%d/%s" % (t + 1, _final_key(key))] = np.array(
                    [digest(_oracle_final(net, key))], np.uint64)
    for k in case.record:
        out["digest/%s/%s" % k] = np.array(dig[k], np.uint64)
        out["count/%s/%s" % k] = np.array(cnt[k], np.int32)
    return out


def run_library(case, syngen, steps=None, extra_args=None, state_file=None, start=0):
    """Runs ``case`` through the drop-in front-end ``syngen`` (either library);
    ``extra_args`` are added to the run arguments.  With ``state_file`` the
    network starts from that saved state (in place of the injections) and
    takes the case's inputs from step ``start`` on."""
    from tests.golden.cases import callback_injections
    steps = case.steps if steps is None else steps
    sizes = case_sizes(case)
    net_dict, injections, weight_arrays, delay_arrays = callback_injections(
        case.net, case.injections(sizes))
    if state_file is not None:
        net_dict, injections = case.net, {}

    def weight_cb(ID, size, weights):
        syngen.FloatArray(size, weights).to_np_array()[:] = weight_arrays[ID]

    def delay_cb(ID, size, weights, delays):
        syngen.IntArray(size, delays).to_np_array()[:] = delay_arrays[ID]

    syngen.create_weight_callback("golden_weight", weight_cb)
    syngen.create_delay_weight_callback("golden_delay", delay_cb)
    net = syngen.Network(net_dict)
    net.build_state()
    if state_file is not None:
        net.load_state(state_file)
    for key, arr in injections.items():
        if key[0] == "neuron":
            dst = net.get_neuron_data(key[1], key[2], key[3]).to_np_array()
        else:
            dst = net.get_weight_matrix(key[1], key[2]).to_np_array()
        assert dst.size == arr.size, (key, dst.size, arr.size)
        dst.view(arr.dtype)[:] = arr
    inputs = case.input_arrays(sizes, start + steps)[start:]
    step = {"in": 0}
    in_layers = sorted(case.inputs)
    rec = {k: [] for k in case.record}

    def in_cb(ID, size, ptr):
        syngen.FloatArray(size, ptr).to_np_array()[:] = inputs[step["in"]][in_layers[ID]]
        if ID == len(in_layers) - 1:
            step["in"] += 1

    def out_cb(ID, size, ptr):
        rec[case.record[ID]].append(syngen.FloatArray(size, ptr).to_np_array().view(np.uint32).copy())

    syngen.create_io_callback("golden_in", in_cb)
    syngen.create_io_callback("golden_out", out_cb)
    modules = []
    structs = {l["name"]: st["name"] for st in case.net["structures"] for l in st["layers"]}
    if in_layers:
        modules.append({"type": "callback", "layers": [
            {"structure": structs[l], "layer": l, "input": True, "function": "golden_in", "id": i}
            for i, l in enumerate(in_layers)]})
    if case.record:
        modules.append({"type": "callback", "layers": [
            {"structure": s, "layer": l, "output": True, "function": "golden_out", "id": i}
            for i, (s, l) in enumerate(case.record)]})
    args = {"iterations": steps, "multithreaded": False, "worker threads": 0,
            "learning flag": case.learning}
    args.update(extra_args or {})
    report = net.run(syngen.Environment({"modules": modules}), args)
    assert report is not None and report.obj is not None, "run failed"
    out = {"rec/%s/%s" % k: np.stack(v) for k, v in rec.items()}
    for key in case.final:
        if key[0] == "neuron":
            arr = net.get_neuron_data(key[1], key[2], key[3])
            out["neuron/%s/%s/%s" % key[1:]] = _as_u32(arr.to_np_array().copy())
        else:
            arr = net.get_weight_matrix(key[1], key[2])
            out["matrix/%s/%s" % key[1:]] = _as_u32(arr.to_np_array().copy())
    return out


def run_digest(case, syngen, steps=None, checkpoints=(), extra_args=None):
    """Runs ``case`` through a drop-in front-end (either library) and keeps
    digests instead of whole records: per step and recorded layer the 64-bit
    digest of the output words and the spike count, and at every checkpoint
    (and the end) the digest of each ``case.final`` array.  The run is split
    into runs of the library at the checkpoints; inputs are drawn step by step
    from the case seed, the same sequence ``Case.input_arrays`` gives."""
    from tests.golden.cases import _rng, callback_injections
    from tests.golden.configs import digest, spike_count
    steps = case.steps if steps is None else steps
    sizes = case_sizes(case)
    net_dict, injections, weight_arrays, delay_arrays = callback_injections(
        case.net, case.injections(sizes))

    def weight_cb(ID, size, weights):
        syngen.FloatArray(size, weights).to_np_array()[:] = weight_arrays[ID]

    def delay_cb(ID, size, weights, delays):
        syngen.IntArray(size, delays).to_np_array()[:] = delay_arrays[ID]

    if not hasattr(syngen, "_delay_weight_callbacks"):
        syngen._delay_weight_callbacks = {}     # the reference front-end never defines it
    syngen.create_weight_callback("golden_weight", weight_cb)
    syngen.create_delay_weight_callback("golden_delay", delay_cb)
    net = syngen.Network(net_dict)
    net.build_state()
    for key, arr in injections.items():
        if key[0] == "neuron":
            dst = net.get_neuron_data(key[1], key[2], key[3]).to_np_array()
        else:
            dst = net.get_weight_matrix(key[1], key[2]).to_np_array()
        assert dst.size == arr.size, (key, dst.size, arr.size)
        dst.view(arr.dtype)[:] = arr
    del injections, weight_arrays, delay_arrays
    rng = _rng(case.seed + 1000)
    in_layers = sorted(case.inputs)
    current = {}
    step = {"in": 0}

    def in_cb(ID, size, ptr):
        if ID == 0:
            current.clear()
            current.update({name: case.inputs[name](rng, step["in"], sizes[name]).astype(np.float32)
                            for name in in_layers})
        syngen.FloatArray(size, ptr).to_np_array()[:] = current[in_layers[ID]]
        if ID == len(in_layers) - 1:
            step["in"] += 1

    dig = {k: [] for k in case.record}
    cnt = {k: [] for k in case.record}

    def out_cb(ID, size, ptr):
        words = syngen.FloatArray(size, ptr).to_np_array().view(np.uint32)
        dig[case.record[ID]].append(digest(words))
        cnt[case.record[ID]].append(spike_count(words))

    syngen.create_io_callback("golden_in", in_cb)
    syngen.create_io_callback("golden_out", out_cb)
    structs = {l["name"]: st["name"] for st in case.net["structures"] for l in st["layers"]}
    modules = []
    if in_layers:
        modules.append({"type": "callback", "layers": [
            {"structure": structs[l], "layer": l, "input": True, "function": "golden_in", "id": i}
            for i, l in enumerate(in_layers)]})
    if case.record:
        modules.append({"type": "callback", "layers": [
            {"structure": s, "layer": l, "output": True, "function": "golden_out", "id": i}
            for i, (s, l) in enumerate(case.record)]})
    env = syngen.Environment({"modules": modules})
    out = {}
    done = 0
    for stop in sorted(set([c for c in checkpoints if 0 < c < steps] + [steps])):
        args = {"iterations": stop - done, "multithreaded": False, "worker threads": 0,
                "learning flag": case.learning}
        args.update(extra_args or {})
        report = net.run(env, args)
        assert report is not None and getattr(report, "obj", report) is not None, "run failed"
        done = stop
        for key in case.final:
            if key[0] == "neuron":
                arr = net.get_neuron_data(key[1], key[2], key[3])
                name = "final@%d/neuron/%s/%s/%s" % ((stop,) + tuple(key[1:]))
            else:
                arr = net.get_weight_matrix(key[1], key[2])
                name = "final@%d/matrix/%s/%s" % ((stop,) + tuple(key[1:]))
            out[name] = np.array([digest(_as_u32(arr.to_np_array()))], np.uint64)
    for (s, l) in case.record:
        out["digest/%s/%s" % (s, l)] = np.array(dig[(s, l)], np.uint64)
        out["count/%s/%s" % (s, l)] = np.array(cnt[(s, l)], np.int32)
    return out


FLOAT_MODELS = ("relay", "rate_encoding")
INT_KEYS = ("output", "time since spike", "delays")


def float_like_keys(case):
    """Result keys holding fp32 values (where any NaN payload counts as equal:
    x86, Arm and the GPU produce different default NaNs)."""
    models = {l["name"]: l["neural model"] for st in case.net["structures"] for l in st["layers"]}
    keys = set()
    for s, l in case.record:
        if models[l] in FLOAT_MODELS:
            keys.add("rec/%s/%s" % (s, l))
    for key in case.final:
        if key[0] == "neuron":
            if key[3] not in INT_KEYS or (key[3] == "output" and models[key[2]] in FLOAT_MODELS):
                keys.add("neuron/%s/%s/%s" % key[1:])
        elif key[2] not in INT_KEYS:
            keys.add("matrix/%s/%s" % key[1:])
    return keys


def compare(got, want, steps=None, tol=None, float_keys=(), nan_keys=()):
    """Bit-exact comparison; keys matching ``float_keys`` use relative tolerance
    ``tol``; in ``nan_keys`` two NaNs match whatever their payload."""
    problems = []
    for k, w in want.items():
        if k not in got:
            problems.append("missing " + k)
            continue
        g = got[k]
        if steps is not None and k.startswith("rec/"):
            w = w[:steps]
        if g.shape != w.shape:
            problems.append("%s shape %s != %s" % (k, g.shape, w.shape))
            continue
        if tol is not None and any(f in k for f in float_keys):
            gf, wf = g.view(np.float32), w.view(np.float32)
            bad = ~np.isclose(gf, wf, rtol=tol, atol=tol, equal_nan=True)
        else:
            bad = g != w
            if k in nan_keys:
                bad &= ~(np.isnan(g.view(np.float32)) & np.isnan(w.view(np.float32)))
        if bad.any():
            idx = np.argwhere(bad)[0]
            problems.append("%s: %d mismatches, first at %s got %r want %r"
                            % (k, int(bad.sum()), tuple(idx), g[tuple(idx)], w[tuple(idx)]))
    return problems


def run_gol_digest(syngen, side=2048, steps=10000, every=1000, extra_args=None):
    """The game_of_life configuration through a drop-in front-end: ``steps``
    timesteps in runs of ``every``; after each run the digests of the board's
    output words and input register."""
    from tests.golden.configs import c1_initial_words, c1_net, digest
    net = syngen.Network(c1_net(side))
    net.build_state()
    net.get_neuron_data("g", "board", "output").to_np_array().view(np.uint32)[:] = \
        c1_initial_words(side)
    env = syngen.Environment({"modules": []})
    words, inputs = [], []
    for _ in range(steps // every):
        args = {"iterations": every, "multithreaded": False, "worker threads": 0,
                "learning flag": False}
        args.update(extra_args or {})
        report = net.run(env, args)
        assert report is not None and getattr(report, "obj", report) is not None, "run failed"
        words.append(digest(net.get_neuron_data("g", "board", "output").to_np_array().view(np.uint32)))
        inputs.append(digest(net.get_neuron_data("g", "board", "input").to_np_array().view(np.uint32)))
    return {"digest/words": np.array(words, np.uint64), "digest/input": np.array(inputs, np.uint64)}
