"""Seeded parity cases shared by the fixture generator and the tests.

Each case is a network in the reference JSON schema plus every random quantity
injected explicitly (the reference's own initialisers are unseedable): weights,
Izhikevich per-synapse state, delays, initial outputs and per-step input
currents.  ``make_golden.py`` runs the reference's CPU library on these cases
and stores what it produced; tests rebuild the same inputs from the seeds.
"""
import numpy as np


def _rng(seed):
    return np.random.default_rng(seed)


class Case:
    def __init__(self, name, net, steps, seed, inject=None, inputs=None, record=(),
                 final=(), learning=True, tol=None):
        self.name = name
        self.net = net
        self.steps = steps
        self.seed = seed
        self.inject = inject or (lambda rng, sizes: {})
        self.inputs = inputs or {}       # layer name -> fn(rng, step, size) -> float32
        self.record = list(record)       # (structure, layer) output word 0 per step
        self.final = list(final)         # ("neuron", structure, layer, key) / ("matrix", conn, key)
        self.learning = learning
        self.tol = tol or {}             # key -> relative tolerance (float paths with libm)

    def input_arrays(self, sizes, steps=None):
        """Per-step input arrays, deterministic in the seed."""
        rng = _rng(self.seed + 1000)
        out = []
        for t in range(self.steps if steps is None else steps):
            out.append({name: fn(rng, t, sizes[name]).astype(np.float32)
                        for name, fn in sorted(self.inputs.items())})
        return out

    def injections(self, sizes):
        return self.inject(_rng(self.seed), sizes)


def callback_injections(net, injections):
    """Moves the injections that must happen while a state is built into
    weight-config callbacks, as the reference's front-end offers them
    (weight_matrix.cpp:853-869, 930-949): ("matrix", c, "init weights") sets
    the dense weights before a sparse connection is compacted, and
    ("matrix", c, "delays") the per-synapse delays.  Returns the rewritten
    network, the remaining injections and {id: array} per callback kind; a
    connection's id is its position in the network."""
    import copy
    net = copy.deepcopy(net)
    rest = dict(injections)
    weights, delays = {}, {}
    for i, c in enumerate(net["connections"]):
        for key, kind, store in ((("matrix", c["name"], "init weights"), "callback", weights),
                                 (("matrix", c["name"], "delays"), "delay callback", delays)):
            if key in rest:
                wc = c.setdefault("weight config", {"type": "flat", "weight": 1.0})
                wc[kind] = "golden_weight" if kind == "callback" else "golden_delay"
                wc["id"] = i
                store[i] = rest.pop(key)
    return net, rest, weights, delays


def _layer(name, model, rows, cols, **kw):
    d = {"name": name, "neural model": model, "rows": rows, "columns": cols}
    d.update(kw)
    return d


def _gol_net(rows, cols, field=3, delay=None, **rule):
    conn = {"name": "nbr", "from layer": "board", "to layer": "board", "type": "convergent",
            "convolutional": True, "plastic": False, "opcode": "add",
            "weight config": {"type": "flat", "weight": 1.0, "diagonal": False},
            "arborized config": {"field size": field, "wrap": True}}
    if delay is not None:
        conn["delay"] = delay
    return {"structures": [{"name": "g", "type": "parallel",
                            "layers": [_layer("board", "game_of_life", rows, cols, **rule)]}],
            "connections": [conn]}


def _gol_inject(p):
    def f(rng, sizes):
        n = sizes["board"]
        alive = (rng.random(n) < p).astype(np.uint32)
        return {("neuron", "g", "board", "output"): alive << np.uint32(31)}
    return f


def _gol_inject_history(p, words):
    def f(rng, sizes):
        n = sizes["board"]
        return {("neuron", "g", "board", "output"):
                rng.integers(0, 2**32, n * words, dtype=np.uint64).astype(np.uint32)}
    return f


def cases():
    out = []

    # --- game of life ---------------------------------------------------
    out.append(Case("gol_16x16", _gol_net(16, 16), 80, 11, inject=_gol_inject(0.3),
                    record=[("g", "board")], final=[("neuron", "g", "board", "output"),
                                                     ("neuron", "g", "board", "input")]))
    out.append(Case("gol_12x20_field5_rules",
                    _gol_net(12, 20, field=5, survival_min=3, survival_max=6,
                             birth_min=4, birth_max=6),
                    40, 12, inject=_gol_inject_history(0.5, 1),
                    record=[("g", "board")], final=[("neuron", "g", "board", "output")]))
    out.append(Case("gol_two_word_history", _gol_net(10, 14, delay=37), 40, 13,
                    inject=_gol_inject_history(0.5, 2),
                    record=[("g", "board")], final=[("neuron", "g", "board", "output")]))

    # --- base activator over every connection type and opcode -----------
    src = _layer("src", "relay", 6, 8)
    net = {"structures": [{"name": "s", "type": "parallel", "layers": [
        src,
        _layer("fc", "relay", 4, 5),
        _layer("sub", "relay", 5, 7, ramp=True),
        _layer("one", "rate_encoding", 6, 8),
        _layer("conv", "relay", 6, 8),
        _layer("conv_s2", "relay", 3, 4),
        _layer("div", "rate_encoding", 12, 16),
        _layer("pool", "relay", 6, 8),
    ]}], "connections": [
        {"name": "c_fc_add", "from layer": "src", "to layer": "fc", "type": "fully connected",
         "opcode": "add", "plastic": False},
        {"name": "c_fc_mult", "from layer": "src", "to layer": "fc", "type": "fully connected",
         "opcode": "mult", "plastic": False},
        {"name": "c_sub_sub", "from layer": "src", "to layer": "sub", "type": "subset",
         "opcode": "sub", "plastic": False,
         "subset config": {"from row start": 1, "from row end": 5, "from column start": 2,
                           "from column end": 7, "to row start": 1, "to row end": 4,
                           "to column start": 0, "to column end": 6}},
        {"name": "c_one_add", "from layer": "src", "to layer": "one", "type": "one to one",
         "opcode": "add", "plastic": False},
        {"name": "c_one_heavi", "from layer": "src", "to layer": "one", "type": "one to one",
         "opcode": "add_heaviside", "plastic": False},
        {"name": "c_conv_nowrap", "from layer": "src", "to layer": "conv", "type": "convergent",
         "opcode": "add", "plastic": False,
         "arborized config": {"field size": 3, "wrap": False}},
        {"name": "c_conv_wrap_sp", "from layer": "src", "to layer": "conv", "type": "convergent",
         "opcode": "sub_heaviside", "plastic": False,
         "arborized config": {"field size": 3, "spacing": 2, "wrap": True}},
        {"name": "c_conv_div", "from layer": "src", "to layer": "conv", "type": "convergent",
         "opcode": "div", "plastic": False, "convolutional": True,
         "arborized config": {"row field size": 2, "column field size": 3, "offset": -1,
                              "wrap": True}},
        {"name": "c_conv_stride2", "from layer": "src", "to layer": "conv_s2", "type": "convergent",
         "opcode": "add", "plastic": False,
         "arborized config": {"field size": 4, "stride": 2, "offset": -1, "wrap": False}},
        {"name": "c_div", "from layer": "src", "to layer": "div", "type": "divergent",
         "opcode": "add", "plastic": False,
         "arborized config": {"field size": 3, "stride": 2, "wrap": False}},
        {"name": "c_div_conv", "from layer": "src", "to layer": "div", "type": "divergent",
         "opcode": "mult_heaviside", "plastic": False, "convolutional": True,
         "arborized config": {"field size": 2, "stride": 2, "wrap": True}},
        {"name": "c_pool", "from layer": "src", "to layer": "pool", "type": "convergent",
         "opcode": "pool", "plastic": False,
         "arborized config": {"field size": 3, "wrap": True}},
    ]}
    base_conns = [c["name"] for c in net["connections"]]

    def inj_base(rng, sizes):
        d = {}
        for name in base_conns:
            n = sizes["conn:" + name]
            d[("matrix", name, "weights")] = rng.uniform(-1.0, 1.0, n).astype(np.float32)
        return d
    out.append(Case("base_all_types", net, 12, 21, inject=inj_base,
                    inputs={"src": lambda rng, t, n: rng.normal(0.0, 1.0, n)},
                    record=[("s", l) for l in ("fc", "sub", "one", "conv", "conv_s2", "div", "pool")],
                    final=[("neuron", "s", l, "input") for l in
                           ("fc", "sub", "one", "conv", "conv_s2", "div", "pool")],
                    tol={"rate_encoding": 2e-7}))

    # --- Izhikevich, the config-0 topology at small size ----------------
    def iz_c0(side, steps, seed, rate, value):
        n = side * side
        net = {"structures": [{"name": "s", "type": "parallel", "layers": [
            _layer("in", "relay", side, side),
            _layer("iz", "izhikevich", side, side, params="regular")]}],
            "connections": [
                {"name": "c_in", "from layer": "in", "to layer": "iz", "type": "convergent",
                 "plastic": False, "opcode": "add",
                 "arborized config": {"field size": 5, "wrap": True}},
                {"name": "c_rec", "from layer": "iz", "to layer": "iz",
                 "type": "fully connected", "plastic": False, "opcode": "sub"}]}

        def inj(rng, sizes):
            nin = sizes["conn:c_in"]
            nrec = sizes["conn:c_rec"]
            v0 = np.full(n, -65.0, np.float32)
            return {("matrix", "c_in", "weights"): rng.uniform(0, 0.5, nin).astype(np.float32),
                    ("matrix", "c_in", "short term w"): np.full(nin, 0.5, np.float32),
                    ("matrix", "c_rec", "weights"):
                        (rng.uniform(0, 0.2, nrec) * (rng.random(nrec) < 0.2)).astype(np.float32),
                    ("matrix", "c_rec", "delays"): rng.integers(0, 4, nrec).astype(np.int32),
                    ("neuron", "s", "iz", "voltage"): v0,
                    ("neuron", "s", "iz", "recovery"): (np.float32(0.2) * v0).astype(np.float32)}
        return Case("iz_c0_%d" % side, net, steps, seed, inject=inj,
                    inputs={"in": lambda rng, t, m: (rng.random(m) < rate) * value},
                    record=[("s", "iz"), ("s", "in")],
                    final=[("neuron", "s", "iz", k) for k in
                           ("voltage", "recovery", "ampa", "nmda", "gabaa", "gabab",
                            "post trace", "time since spike", "output", "dopamine")]
                    + [("matrix", "c_in", k) for k in ("short trace", "long trace", "time since spike")]
                    + [("matrix", "c_rec", k) for k in ("short trace", "long trace", "time since spike")])
    out.append(iz_c0(8, 300, 31, 0.05, 1.0))
    out.append(iz_c0(32, 120, 32, 0.01, 1.0))

    # --- Izhikevich plasticity (STDP + STP), every plastic connection type --
    net = {"structures": [{"name": "s", "type": "parallel", "layers": [
        _layer("in", "relay", 8, 8),
        _layer("e", "izhikevich", 8, 8, params="regular"),
        _layer("i", "izhikevich", 6, 6, params="fast")]}],
        "connections": [
            {"name": "p_conv", "from layer": "in", "to layer": "e", "type": "convergent",
             "opcode": "add", "arborized config": {"field size": 3, "wrap": True}},
            {"name": "p_ee", "from layer": "e", "to layer": "e", "type": "fully connected",
             "opcode": "add", "max weight": 0.5, "learning rate": 0.05},
            {"name": "p_ie", "from layer": "i", "to layer": "e", "type": "fully connected",
             "opcode": "sub"},
            {"name": "p_ei", "from layer": "e", "to layer": "i", "type": "subset", "opcode": "add",
             "subset config": {"from row start": 0, "from row end": 6, "from column start": 1,
                               "from column end": 7, "to row start": 0, "to row end": 5,
                               "to column start": 0, "to column end": 6}},
            {"name": "p_div", "from layer": "i", "to layer": "e", "type": "divergent",
             "opcode": "add", "arborized config": {"field size": 3, "stride": 1}},
            {"name": "p_one", "from layer": "e", "to layer": "e", "type": "one to one",
             "opcode": "sub", "short term plasticity": False}]}
    pconns = ["p_conv", "p_ee", "p_ie", "p_ei", "p_div", "p_one"]

    def inj_plastic(rng, sizes):
        d = {}
        for name in pconns:
            n = sizes["conn:" + name]
            d[("matrix", name, "weights")] = rng.uniform(0.0, 0.6, n).astype(np.float32)
            d[("matrix", name, "short term w")] = rng.uniform(0.2, 0.6, n).astype(np.float32)
            d[("matrix", name, "delays")] = rng.integers(0, 5, n).astype(np.int32)
        return d
    finals = []
    for name in pconns:
        finals += [("matrix", name, k) for k in ("weights", "presyn trace", "weight derivatives",
                                                 "short term R", "short term w", "short trace",
                                                 "long trace", "time since spike")]
    finals += [("neuron", "s", l, k) for l in ("e", "i")
               for k in ("voltage", "recovery", "post trace", "time since spike", "output")]
    out.append(Case("iz_plastic", net, 150, 41, inject=inj_plastic,
                    inputs={"in": lambda rng, t, m: (rng.random(m) < 0.15) * 2.0},
                    record=[("s", "e"), ("s", "i")], final=finals,
                    tol={"istdp": 0.0}))

    # --- Izhikevich subset / fully connected matrices wide enough for the
    #     column kernels (destination counts divisible by 4) ----------------
    net = {"structures": [{"name": "s", "type": "parallel", "layers": [
        _layer("in", "relay", 12, 16),
        _layer("a", "izhikevich", 12, 16, params="regular"),
        _layer("b", "izhikevich", 10, 20, params="fast")]}],
        "connections": [
            {"name": "q_in", "from layer": "in", "to layer": "a", "type": "fully connected",
             "opcode": "add", "plastic": False},
            {"name": "q_ab", "from layer": "a", "to layer": "b", "type": "subset", "opcode": "add",
             "learning rate": 0.02,
             "subset config": {"from row start": 2, "from row end": 10, "from column start": 3,
                               "from column end": 15, "to row start": 1, "to row end": 9,
                               "to column start": 4, "to column end": 16}},
            {"name": "q_ba", "from layer": "b", "to layer": "a", "type": "subset", "opcode": "sub",
             "subset config": {"from row start": 0, "from row end": 10, "from column start": 0,
                               "from column end": 20, "to row start": 0, "to row end": 12,
                               "to column start": 0, "to column end": 16}},
            {"name": "q_bb", "from layer": "b", "to layer": "b", "type": "fully connected",
             "opcode": "mult", "plastic": False}]}
    qconns = ["q_in", "q_ab", "q_ba", "q_bb"]

    def inj_q(rng, sizes):
        d = {}
        for name in qconns:
            n = sizes["conn:" + name]
            d[("matrix", name, "weights")] = rng.uniform(0.0, 0.12, n).astype(np.float32)
            d[("matrix", name, "short term w")] = rng.uniform(0.3, 0.7, n).astype(np.float32)
            d[("matrix", name, "delays")] = rng.integers(0, 6, n).astype(np.int32)
        return d
    qfinal = []
    for name in qconns:
        qfinal += [("matrix", name, k) for k in ("weights", "short trace", "long trace",
                                                 "time since spike", "short term R",
                                                 "short term w", "weight derivatives",
                                                 "presyn trace")]
    qfinal += [("neuron", "s", l, k) for l in ("a", "b")
               for k in ("voltage", "recovery", "output", "mult", "time since spike")]
    out.append(Case("iz_subset_columns", net, 120, 61, inject=inj_q,
                    inputs={"in": lambda rng, t, m: (rng.random(m) < 0.1) * 1.0},
                    record=[("s", "a"), ("s", "b")], final=qfinal))

    # --- Izhikevich opcodes: mult, reward, gap, direct, default delays,
    #     multi-word BIT history read by a FLOAT layer ----------------------
    net = {"structures": [{"name": "s", "type": "parallel", "layers": [
        _layer("in", "relay", 6, 6),
        _layer("iz", "izhikevich", 6, 6, params="chattering", **{"neuron spacing": 0.3}),
        _layer("ro", "relay", 6, 6)]}],
        "connections": [
            {"name": "o_drive", "from layer": "in", "to layer": "iz", "type": "one to one",
             "opcode": "add", "plastic": False},
            {"name": "o_direct", "from layer": "in", "to layer": "iz", "type": "convergent",
             "opcode": "add", "plastic": False, "direct": True,
             "arborized config": {"field size": 3, "wrap": True}},
            {"name": "o_mult", "from layer": "iz", "to layer": "iz", "type": "fully connected",
             "opcode": "mult", "plastic": False},
            {"name": "o_reward", "from layer": "in", "to layer": "iz", "type": "fully connected",
             "opcode": "reward", "plastic": False},
            {"name": "o_gap", "from layer": "iz", "to layer": "iz", "type": "fully connected",
             "opcode": "gap", "plastic": False},
            {"name": "o_rec", "from layer": "iz", "to layer": "iz", "type": "fully connected",
             "opcode": "add", "plastic": False},
            {"name": "o_read", "from layer": "iz", "to layer": "ro", "type": "one to one",
             "opcode": "add", "plastic": False, "delay": 45}]}

    def inj_ops(rng, sizes):
        d = {}
        for name in ("o_drive", "o_mult", "o_reward", "o_rec"):
            n = sizes["conn:" + name]
            d[("matrix", name, "weights")] = rng.uniform(0.0, 0.3, n).astype(np.float32)
            d[("matrix", name, "short term w")] = rng.uniform(0.3, 0.7, n).astype(np.float32)
        d[("matrix", "o_drive", "weights")] = np.full(sizes["conn:o_drive"], 1.0, np.float32)
        d[("matrix", "o_direct", "weights")] = rng.uniform(0.0, 2.0, sizes["conn:o_direct"]).astype(np.float32)
        d[("matrix", "o_gap", "weights")] = rng.uniform(0.0, 0.02, sizes["conn:o_gap"]).astype(np.float32)
        return d
    out.append(Case("iz_opcodes", net, 200, 51, inject=inj_ops,
                    inputs={"in": lambda rng, t, m: (rng.random(m) < 0.2) * 3.0},
                    record=[("s", "iz"), ("s", "ro")],
                    final=[("neuron", "s", "iz", k) for k in
                           ("voltage", "recovery", "mult", "dopamine", "input", "output")]
                    + [("neuron", "s", "ro", "output")]))

    # --- dendritic trees ---------------------------------------------------
    # Registers: tree a=1, a1=2, a2=3, b=4, c=5; rtree h=1, g=2; board n=1;
    # iz m=1.  Root-level connections listed first still run after the
    # internal subtrees (post-order walk).
    conv3 = {"field size": 3, "wrap": False}
    net = {"structures": [{"name": "d", "type": "parallel", "layers": [
        _layer("src", "relay", 6, 8),
        _layer("aux", "relay", 6, 8),
        _layer("tree", "relay", 6, 8, dendrites=[
            {"name": "a", "opcode": "mult", "init": 1.0, "children": [
                {"name": "a1", "opcode": "add"},
                {"name": "a2", "opcode": "sub", "init": 0.5}]},
            {"name": "b", "opcode": "sub"},
            {"name": "c", "opcode": "pool", "init": -2.0}]),
        _layer("rtree", "rate_encoding", 4, 5, dendrites=[
            {"name": "h", "opcode": "mult_heaviside", "init": 0.25},
            {"name": "g", "opcode": "div", "init": 2.0}]),
        _layer("board", "game_of_life", 12, 12, dendrites=[{"name": "n", "opcode": "add"}]),
        _layer("iz", "izhikevich", 6, 8, dendrites=[{"name": "m", "opcode": "mult", "init": 1.0}]),
    ]}], "connections": [
        {"name": "t_root", "from layer": "src", "to layer": "tree", "type": "one to one",
         "opcode": "add", "plastic": False},
        {"name": "t_a", "from layer": "src", "to layer": "tree", "type": "convergent",
         "opcode": "add", "plastic": False, "dendrite": "a", "arborized config": conv3},
        {"name": "t_a1", "from layer": "aux", "to layer": "tree", "type": "fully connected",
         "opcode": "add", "plastic": False, "dendrite": "a1"},
        {"name": "t_a2", "from layer": "src", "to layer": "tree", "type": "one to one",
         "opcode": "mult", "plastic": False, "dendrite": "a2"},
        {"name": "t_a1b", "from layer": "aux", "to layer": "tree", "type": "convergent",
         "opcode": "sub", "plastic": False, "dendrite": "a1",
         "arborized config": {"field size": 3, "wrap": True}},
        {"name": "t_b", "from layer": "src", "to layer": "tree", "type": "convergent",
         "convolutional": True, "opcode": "add", "plastic": False, "dendrite": "b",
         "arborized config": {"field size": 3, "wrap": True}},
        {"name": "t_c", "from layer": "aux", "to layer": "tree", "type": "one to one",
         "opcode": "add", "plastic": False, "dendrite": "c"},
        {"name": "t_root2", "from layer": "aux", "to layer": "tree", "type": "one to one",
         "opcode": "sub", "plastic": False},
        {"name": "r_h", "from layer": "src", "to layer": "rtree", "type": "fully connected",
         "opcode": "add", "plastic": False, "dendrite": "h"},
        {"name": "r_g", "from layer": "aux", "to layer": "rtree", "type": "subset",
         "opcode": "add", "plastic": False, "dendrite": "g",
         "subset config": {"from row start": 0, "from row end": 3, "from column start": 1,
                           "from column end": 5, "to row start": 1, "to row end": 3,
                           "to column start": 0, "to column end": 4}},
        {"name": "r_root", "from layer": "src", "to layer": "rtree", "type": "fully connected",
         "opcode": "add", "plastic": False},
        {"name": "nbr", "from layer": "board", "to layer": "board", "type": "convergent",
         "convolutional": True, "plastic": False, "opcode": "add", "dendrite": "n",
         "weight config": {"type": "flat", "weight": 1.0, "diagonal": False},
         "arborized config": {"field size": 3, "wrap": True}},
        {"name": "i_drive", "from layer": "src", "to layer": "iz", "type": "one to one",
         "opcode": "add", "plastic": False, "direct": True},
        {"name": "i_gate", "from layer": "aux", "to layer": "iz", "type": "one to one",
         "opcode": "mult", "plastic": False, "direct": True, "dendrite": "m"},
        {"name": "i_trace", "from layer": "board", "to layer": "iz", "type": "fully connected",
         "opcode": "add", "plastic": False, "dendrite": "m"},
    ]}
    dend_conns = [c["name"] for c in net["connections"] if c["name"] not in ("nbr",)]

    def inj_dend(rng, sizes):
        d = {}
        for name in dend_conns:
            n = sizes["conn:" + name]
            d[("matrix", name, "weights")] = rng.uniform(-1.0, 1.0, n).astype(np.float32)
        d[("matrix", "i_drive", "weights")] = rng.uniform(5.0, 25.0, sizes["conn:i_drive"]).astype(np.float32)
        d[("matrix", "i_gate", "weights")] = rng.uniform(0.0, 2.0, sizes["conn:i_gate"]).astype(np.float32)
        d[("matrix", "i_trace", "weights")] = rng.uniform(0.0, 0.01, sizes["conn:i_trace"]).astype(np.float32)
        # whole history words: bit 0 (the rule's "previously alive") random too
        d[("neuron", "d", "board", "output")] = rng.integers(0, 2**32, sizes["board"],
                                                             dtype=np.uint64).astype(np.uint32)
        return d
    out.append(Case("dendrites", net, 16, 71, inject=inj_dend,
                    inputs={"src": lambda rng, t, n: rng.normal(0.0, 1.0, n),
                            "aux": lambda rng, t, n: rng.normal(0.0, 1.0, n)},
                    record=[("d", l) for l in ("tree", "rtree", "board", "iz")],
                    final=[("neuron", "d", l, "input") for l in ("tree", "rtree", "board", "iz")]
                    + [("neuron", "d", "iz", k) for k in ("voltage", "recovery", "post trace")]
                    + [("matrix", "i_trace", "short term R")]))

    # --- second-order nodes --------------------------------------------------
    # so_fc: host + two slaves on g (register 1, not initialised at build);
    # so_mix: second-order q inside p, and a convolutional host/slave pair on
    # k; so_sub: subset host and slave of different window shapes.
    net = {"structures": [{"name": "o", "type": "parallel", "layers": [
        _layer("src", "relay", 6, 8),
        _layer("mod", "relay", 6, 8),
        _layer("m9", "relay", 3, 3),
        _layer("so_fc", "relay", 4, 5, dendrites=[
            {"name": "g", "second order": True, "opcode": "add", "init": 0.25}]),
        _layer("so_mix", "relay", 6, 8, dendrites=[
            {"name": "p", "opcode": "add", "init": 1.0, "children": [
                {"name": "q", "second order": True, "opcode": "mult", "init": 1.0}]},
            {"name": "k", "second order": True, "opcode": "sub"}]),
        _layer("so_sub", "relay", 4, 6, dendrites=[{"name": "s", "second order": True}]),
    ]}], "connections": [
        {"name": "fc_host", "from layer": "src", "to layer": "so_fc", "type": "fully connected",
         "opcode": "add", "plastic": False, "dendrite": "g"},
        {"name": "fc_slave1", "from layer": "mod", "to layer": "so_fc", "type": "fully connected",
         "opcode": "mult", "plastic": False, "dendrite": "g"},
        {"name": "fc_slave2", "from layer": "src", "to layer": "so_fc", "type": "fully connected",
         "opcode": "add", "plastic": False, "dendrite": "g"},
        {"name": "fc_root", "from layer": "mod", "to layer": "so_fc", "type": "fully connected",
         "opcode": "add", "plastic": False},
        {"name": "q_host", "from layer": "src", "to layer": "so_mix", "type": "convergent",
         "opcode": "add", "plastic": False, "dendrite": "q",
         "arborized config": {"field size": 3, "wrap": True}},
        {"name": "q_slave", "from layer": "mod", "to layer": "so_mix", "type": "convergent",
         "opcode": "mult", "plastic": False, "dendrite": "q", "arborized config": conv3},
        {"name": "p_leaf", "from layer": "mod", "to layer": "so_mix", "type": "one to one",
         "opcode": "add", "plastic": False, "dendrite": "p"},
        {"name": "k_host", "from layer": "src", "to layer": "so_mix", "type": "convergent",
         "convolutional": True, "opcode": "add", "plastic": False, "dendrite": "k",
         "arborized config": {"field size": 3, "wrap": True}},
        {"name": "k_slave", "from layer": "m9", "to layer": "so_mix", "type": "convergent",
         "convolutional": True, "opcode": "mult", "plastic": False, "dendrite": "k",
         "arborized config": {"field size": 3, "stride": 0, "spacing": 1}},
        {"name": "s_host", "from layer": "src", "to layer": "so_sub", "type": "subset",
         "opcode": "add", "plastic": False, "dendrite": "s",
         "subset config": {"from row start": 0, "from row end": 2, "from column start": 0,
                           "from column end": 4, "to row start": 0, "to row end": 2,
                           "to column start": 0, "to column end": 3}},
        {"name": "s_slave", "from layer": "mod", "to layer": "so_sub", "type": "subset",
         "opcode": "add", "plastic": False, "dendrite": "s",
         "subset config": {"from row start": 1, "from row end": 5, "from column start": 2,
                           "from column end": 5, "to row start": 1, "to row end": 3,
                           "to column start": 2, "to column end": 4}},
    ]}
    so_conns = [c["name"] for c in net["connections"]]

    def inj_so(rng, sizes):
        d = {}
        for name in so_conns:
            n = sizes["conn:" + name]
            lo, hi = (0.5, 1.5) if name in ("fc_slave1", "q_slave", "k_slave") else (-1.0, 1.0)
            d[("matrix", name, "weights")] = rng.uniform(lo, hi, n).astype(np.float32)
        return d
    out.append(Case("second_order", net, 12, 81, inject=inj_so,
                    inputs={"src": lambda rng, t, n: rng.normal(0.0, 1.0, n),
                            "mod": lambda rng, t, n: rng.normal(0.0, 1.0, n),
                            "m9": lambda rng, t, n: rng.normal(1.0, 0.5, n)},
                    record=[("o", l) for l in ("so_fc", "so_mix", "so_sub")],
                    final=[("neuron", "o", l, "input") for l in ("so_fc", "so_mix", "so_sub")]
                    + [("matrix", c, "weights") for c in ("fc_host", "q_host", "k_host", "s_host")]))

    # --- sparse connections --------------------------------------------------
    # Dense weights with zeros go in through a weight callback before the
    # state compacts them: fully connected, wrapping and clipped convergent,
    # divergent, subset (its window rows serve the layer's first
    # destinations, as in the reference), one to one, an all-zero matrix,
    # and plastic / non-plastic Izhikevich connections with distance delays.
    net = {"structures": [{"name": "p", "type": "parallel", "layers": [
        _layer("src", "relay", 6, 8),
        _layer("sfc", "relay", 5, 6),
        _layer("sconv", "relay", 6, 8),
        _layer("sdiv", "rate_encoding", 12, 16),
        _layer("ssub", "relay", 4, 6),
        _layer("sone", "relay", 6, 8),
        _layer("iz_in", "relay", 8, 8),
        _layer("iz", "izhikevich", 8, 8),
    ]}], "connections": [
        {"name": "p_fc", "from layer": "src", "to layer": "sfc", "type": "fully connected",
         "opcode": "add", "plastic": False, "sparse": True},
        {"name": "p_conv_wrap", "from layer": "src", "to layer": "sconv", "type": "convergent",
         "opcode": "add", "plastic": False, "sparse": True,
         "arborized config": {"field size": 3, "wrap": True}},
        {"name": "p_conv_clip", "from layer": "src", "to layer": "sconv", "type": "convergent",
         "opcode": "sub", "plastic": False, "sparse": True,
         "arborized config": {"field size": 5, "spacing": 2, "wrap": False}},
        {"name": "p_div", "from layer": "src", "to layer": "sdiv", "type": "divergent",
         "opcode": "add", "plastic": False, "sparse": True,
         "arborized config": {"field size": 3, "stride": 2, "wrap": True}},
        {"name": "p_sub", "from layer": "src", "to layer": "ssub", "type": "subset",
         "opcode": "add", "plastic": False, "sparse": True,
         "subset config": {"from row start": 1, "from row end": 5, "from column start": 2,
                           "from column end": 7, "to row start": 1, "to row end": 4,
                           "to column start": 2, "to column end": 6}},
        {"name": "p_one", "from layer": "src", "to layer": "sone", "type": "one to one",
         "opcode": "add", "plastic": False, "sparse": True},
        {"name": "p_zero", "from layer": "src", "to layer": "sone", "type": "fully connected",
         "opcode": "sub", "plastic": False, "sparse": True},
        {"name": "i_drive", "from layer": "iz_in", "to layer": "iz", "type": "one to one",
         "opcode": "add", "plastic": False, "direct": True},
        {"name": "i_ff", "from layer": "iz_in", "to layer": "iz", "type": "fully connected",
         "opcode": "add", "plastic": False, "sparse": True},
        {"name": "i_rec", "from layer": "iz", "to layer": "iz", "type": "convergent",
         "opcode": "add", "plastic": True, "sparse": True, "max weight": 0.5,
         "arborized config": {"field size": 5, "wrap": True}},
    ]}
    sparse_conns = [c["name"] for c in net["connections"] if c.get("sparse")]

    def inj_sparse(rng, sizes):
        d = {}
        for name in sparse_conns:
            n = sizes["dense:" + name]
            w = rng.uniform(-1.0, 1.0, n).astype(np.float32)
            if name in ("i_ff", "i_rec"):
                w = np.abs(w) * np.float32(0.02 if name == "i_ff" else 0.3)
            w[rng.random(n) < 0.5] = 0.0
            if name == "p_zero":
                w[:] = 0.0
            d[("matrix", name, "init weights")] = w
        d[("matrix", "i_drive", "weights")] = np.full(64, 1.0, np.float32)
        return d
    out.append(Case("sparse", net, 60, 91, inject=inj_sparse,
                    inputs={"src": lambda rng, t, n: rng.normal(0.0, 1.0, n),
                            "iz_in": lambda rng, t, n: (rng.random(n) < 0.15) * 12.0},
                    record=[("p", l) for l in ("sfc", "sconv", "sdiv", "ssub", "sone", "iz")],
                    final=[("neuron", "p", l, "input") for l in ("sfc", "sconv", "sdiv", "ssub", "sone")]
                    + [("neuron", "p", "iz", k) for k in ("voltage", "recovery", "post trace")]
                    + [("matrix", c, k) for c in ("i_rec", "i_ff")
                       for k in ("weights", "short term w", "short term R", "presyn trace")]
                    + [("matrix", c, "weights") for c in ("p_fc", "p_div", "p_sub", "p_zero")]))

    # --- the smaller neural models -----------------------------------------
    # binary threshold, hebbian rate encoding (its rule is never applied by
    # the reference), perceptron, sine generator, vp_max.
    net = {"structures": [{"name": "m", "type": "parallel", "layers": [
        _layer("src", "relay", 6, 8),
        _layer("bt", "binary threshold", 6, 8),
        _layer("hb", "hebbian_rate_encoding", 6, 8),
        _layer("pc", "perceptron", 4, 5),
        _layer("sg", "sine generator", 6, 8, frequency=37),
        _layer("vm", "vp_max", 6, 8),
    ]}], "connections": [
        {"name": "m_bt", "from layer": "src", "to layer": "bt", "type": "one to one",
         "opcode": "add", "plastic": False},
        {"name": "m_hb", "from layer": "src", "to layer": "hb", "type": "fully connected",
         "opcode": "add", "plastic": True},
        {"name": "m_pc", "from layer": "src", "to layer": "pc", "type": "fully connected",
         "opcode": "add", "plastic": False},
        {"name": "m_pc_sub", "from layer": "bt", "to layer": "pc", "type": "subset",
         "opcode": "sub", "plastic": False,
         "subset config": {"from row start": 0, "from row end": 3, "from column start": 1,
                           "from column end": 5, "to row start": 1, "to row end": 3,
                           "to column start": 0, "to column end": 4}},
        {"name": "m_sg", "from layer": "src", "to layer": "sg", "type": "one to one",
         "opcode": "add", "plastic": False},
        {"name": "m_vm", "from layer": "src", "to layer": "vm", "type": "convergent",
         "opcode": "add", "plastic": False, "arborized config": {"field size": 3, "wrap": True}},
        {"name": "m_vm_sub", "from layer": "bt", "to layer": "vm", "type": "one to one",
         "opcode": "sub", "plastic": False},
    ]}
    model_conns = [c["name"] for c in net["connections"]]

    def inj_models(rng, sizes):
        return {("matrix", name, "weights"): rng.uniform(-1.0, 1.0, sizes["conn:" + name]).astype(np.float32)
                for name in model_conns}
    out.append(Case("models", net, 40, 101, inject=inj_models,
                    inputs={"src": lambda rng, t, n: rng.normal(0.0, 1.0, n)},
                    record=[("m", l) for l in ("bt", "hb", "pc", "sg", "vm")],
                    final=[("neuron", "m", l, "input") for l in ("bt", "hb", "pc", "sg", "vm")]
                    + [("matrix", "m_hb", "weights")]))

    # --- spnet (Izhikevich's polychronization network) ---------------------
    # Excitatory layer with recurrent STDP ("add") and inhibitory feedback
    # with inverse STDP ("sub"), distance delays, a Poisson-like drive.
    net = {"structures": [{"name": "n", "type": "parallel", "layers": [
        _layer("in", "relay", 10, 10),
        _layer("exc", "spnet", 10, 10, params="regular"),
        _layer("inh", "spnet", 5, 5, params="fast"),
    ]}], "connections": [
        {"name": "n_drive", "from layer": "in", "to layer": "exc", "type": "one to one",
         "opcode": "add", "plastic": False},
        {"name": "n_rec", "from layer": "exc", "to layer": "exc", "type": "convergent",
         "opcode": "add", "plastic": True, "max weight": 10.0,
         "arborized config": {"field size": 5, "wrap": True}},
        {"name": "n_ei", "from layer": "exc", "to layer": "inh", "type": "convergent",
         "opcode": "add", "plastic": False,
         "arborized config": {"field size": 3, "stride": 2, "wrap": True}},
        {"name": "n_ie", "from layer": "inh", "to layer": "exc", "type": "fully connected",
         "opcode": "sub", "plastic": True, "max weight": 5.0},
        {"name": "n_sp", "from layer": "exc", "to layer": "exc", "type": "convergent",
         "opcode": "add", "plastic": True, "max weight": 8.0, "sparse": True,
         "arborized config": {"field size": 3, "wrap": True}},
        {"name": "n_isp", "from layer": "inh", "to layer": "exc", "type": "fully connected",
         "opcode": "sub", "plastic": True, "max weight": 4.0, "sparse": True},
    ]}

    def inj_spnet(rng, sizes):
        d = {
            ("matrix", "n_drive", "weights"): np.full(sizes["conn:n_drive"], 20.0, np.float32),
            ("matrix", "n_rec", "weights"): rng.uniform(0.0, 6.0, sizes["conn:n_rec"]).astype(np.float32),
            ("matrix", "n_ei", "weights"): rng.uniform(0.0, 20.0, sizes["conn:n_ei"]).astype(np.float32),
            ("matrix", "n_ie", "weights"): rng.uniform(0.0, 4.0, sizes["conn:n_ie"]).astype(np.float32),
        }
        for name, hi in (("n_sp", 6.0), ("n_isp", 3.0)):   # sparse: half the weights zero
            w = rng.uniform(0.0, hi, sizes["dense:" + name]).astype(np.float32)
            w[rng.random(w.size) < 0.5] = 0.0
            d[("matrix", name, "init weights")] = w
        return d
    out.append(Case("spnet", net, 200, 111, inject=inj_spnet,
                    inputs={"in": lambda rng, t, n: (rng.random(n) < 0.25) * 1.0},
                    record=[("n", "exc"), ("n", "inh")],
                    final=[("neuron", "n", "exc", k) for k in
                           ("voltage", "recovery", "post trace", "time since spike", "input")]
                    + [("neuron", "n", "inh", k) for k in ("voltage", "recovery")]
                    + [("matrix", c, k) for c in ("n_rec", "n_ie", "n_sp", "n_isp")
                       for k in ("weights", "presyn trace", "weight derivative", "time since spike")]))

    # --- oscillator and self-organising map --------------------------------
    net = {"structures": [{"name": "o", "type": "parallel", "layers": [
        _layer("src", "relay", 6, 8),
        _layer("mod", "relay", 4, 4),
        _layer("osc", "oscillator", 6, 8, tonic=0.2, tau=0.3, decay=0.2),
        _layer("som", "som", 5, 5, **{"rbf scale": 0.002}),
    ]}], "connections": [
        {"name": "o_conv", "from layer": "src", "to layer": "osc", "type": "convergent",
         "opcode": "add", "plastic": False, "arborized config": {"field size": 3, "wrap": True}},
        {"name": "o_one", "from layer": "src", "to layer": "osc", "type": "one to one",
         "opcode": "sub", "plastic": False},
        {"name": "s_fc", "from layer": "src", "to layer": "som", "type": "fully connected",
         "opcode": "add", "plastic": True, "learning rate": 0.05, "neighborhood size": 1},
        {"name": "s_mod", "from layer": "mod", "to layer": "som", "type": "fully connected",
         "opcode": "modulate", "plastic": False},
    ]}

    def inj_osc_som(rng, sizes):
        return {
            ("matrix", "o_conv", "weights"): rng.uniform(-1.0, 1.0, sizes["conn:o_conv"]).astype(np.float32),
            ("matrix", "o_one", "weights"): rng.uniform(-1.0, 1.0, sizes["conn:o_one"]).astype(np.float32),
            ("matrix", "s_fc", "weights"): rng.uniform(-1.0, 1.0, sizes["conn:s_fc"]).astype(np.float32),
            ("matrix", "s_mod", "weights"): rng.uniform(0.0, 0.2, sizes["conn:s_mod"]).astype(np.float32),
        }
    out.append(Case("oscillator_som", net, 40, 121, inject=inj_osc_som,
                    inputs={"src": lambda rng, t, n: rng.normal(0.0, 1.0, n),
                            "mod": lambda rng, t, n: rng.uniform(0.0, 1.0, n)},
                    record=[("o", "osc"), ("o", "som")],
                    final=[("neuron", "o", "osc", k) for k in ("state", "bold", "input")]
                    + [("neuron", "o", "som", k) for k in ("plasticity", "input")]
                    + [("matrix", "s_fc", k) for k in ("weights", "output cache")]))

    # --- neural virtual machine models ------------------------------------
    # Gate connections (decay, then activity gate, learning gate) from a
    # control layer; plain, gated, context and plastic connections into nvm;
    # nvm_heaviside; nvm_compare learning its true state.
    def window(r0, r1, c0, c1):
        return {"from row start": 0, "from row end": 1, "from column start": c0,
                "from column end": c1, "to row start": r0, "to row end": r1,
                "to column start": 0, "to column end": 4}
    net = {"structures": [{"name": "v", "type": "parallel", "layers": [
        _layer("ctl", "relay", 1, 6),
        _layer("x", "relay", 4, 4),
        _layer("mem", "nvm", 4, 4),
        _layer("hv", "nvm_heaviside", 4, 4, gain=2.0),
        _layer("cmp", "nvm_compare", 4, 4, tolerance=0.75),
    ]}], "connections": [
        {"name": "v_decay", "from layer": "ctl", "to layer": "mem", "type": "subset", "decay": True,
         "plastic": False, "subset config": window(0, 1, 0, 1)},
        {"name": "v_gate", "from layer": "ctl", "to layer": "mem", "type": "subset", "gate": True,
         "plastic": False, "subset config": window(0, 2, 1, 3)},
        {"name": "v_learn", "from layer": "ctl", "to layer": "mem", "type": "subset", "learning": True,
         "plastic": False, "subset config": window(1, 4, 3, 4)},
        {"name": "v_plain", "from layer": "x", "to layer": "mem", "type": "one to one",
         "opcode": "add", "plastic": False},
        {"name": "v_ctx", "from layer": "x", "to layer": "mem", "type": "one to one",
         "context": True, "plastic": False},
        {"name": "v_gated", "from layer": "x", "to layer": "mem", "type": "fully connected",
         "gated": True, "plastic": False},
        {"name": "v_rec", "from layer": "mem", "to layer": "mem", "type": "fully connected",
         "plastic": True, "norm": 2.0},
        {"name": "h_in", "from layer": "x", "to layer": "hv", "type": "convergent", "plastic": False,
         "arborized config": {"field size": 3, "wrap": True}},
        {"name": "h_gated", "from layer": "mem", "to layer": "hv", "type": "one to one",
         "gated": True, "plastic": False},
        {"name": "c_gate", "from layer": "ctl", "to layer": "cmp", "type": "subset", "gate": True,
         "plastic": False, "subset config": window(0, 1, 4, 5)},
        {"name": "c_learn", "from layer": "ctl", "to layer": "cmp", "type": "subset", "learning": True,
         "plastic": False, "subset config": window(0, 1, 5, 6)},
        {"name": "c_plastic", "from layer": "x", "to layer": "cmp", "type": "fully connected",
         "plastic": True, "norm": 4.0},
    ]}
    nvm_conns = [c["name"] for c in net["connections"]]

    def inj_nvm(rng, sizes):
        d = {("matrix", n, "weights"): rng.uniform(-1.0, 1.0, sizes["conn:" + n]).astype(np.float32)
             for n in nvm_conns}
        d[("neuron", "v", "cmp", "true_state")] = np.where(rng.random(16) < 0.5, -1.0, 1.0).astype(np.float32)
        return d
    out.append(Case("nvm", net, 40, 131, inject=inj_nvm,
                    inputs={"ctl": lambda rng, t, n: (rng.random(n) < 0.6) * 1.0,
                            "x": lambda rng, t, n: rng.normal(0.0, 1.0, n)},
                    record=[("v", "mem"), ("v", "hv"), ("v", "cmp")],
                    final=[("neuron", "v", "mem", k) for k in ("state", "context", "input")]
                    + [("neuron", "v", "hv", k) for k in ("state", "input")]
                    + [("neuron", "v", "cmp", "input")]
                    + [("matrix", c, "weights") for c in ("v_rec", "c_plastic")]))

    # --- sequential, feedforward and parallel structures ---------------------
    # seq: layers step in dependency order (h2 -> h1 is recurrent, so it reads
    # last step's h2); ff: feedforward, whose updaters read the sources'
    # outputs (perceptron, oscillator, vp_max, sample learn); par: parallel,
    # with an input layer that activates after the sequential structure.
    net = {"structures": [
        {"name": "seq", "type": "sequential", "layers": [
            _layer("out", "relay", 4, 4), _layer("h2", "relay", 4, 4),
            _layer("in", "relay", 4, 4), _layer("h1", "relay", 4, 4, ramp=True)]},
        {"name": "ff", "type": "feedforward", "layers": [
            _layer("x", "relay", 4, 4), _layer("p", "perceptron", 3, 3),
            _layer("o", "oscillator", 4, 4), _layer("v", "vp_max", 4, 4),
            _layer("sp", "sample", 4, 4), _layer("bp", "backprop_rate_encoding", 4, 4)]},
        {"name": "par", "type": "parallel", "layers": [
            _layer("q", "relay", 4, 4), _layer("r", "relay", 4, 4), _layer("z", "relay", 4, 4)]},
    ], "connections": [
        {"name": "s_in", "from layer": "in", "to layer": "h1", "type": "one to one", "plastic": False},
        {"name": "s_12", "from layer": "h1", "to layer": "h2", "type": "fully connected", "plastic": False},
        {"name": "s_back", "from layer": "h2", "to layer": "h1", "type": "one to one", "plastic": False,
         "recurrent": True, "opcode": "sub"},
        {"name": "s_out", "from layer": "h2", "to layer": "out", "type": "one to one", "plastic": False},
        {"name": "f_p", "from layer": "x", "to layer": "p", "type": "fully connected", "plastic": True},
        {"name": "f_o", "from layer": "x", "to layer": "o", "type": "one to one", "plastic": True},
        {"name": "f_v", "from layer": "x", "to layer": "v", "type": "convergent", "plastic": True,
         "arborized config": {"field size": 3, "wrap": True}},
        {"name": "f_sp", "from layer": "x", "to layer": "sp", "type": "one to one", "plastic": True,
         "connection variable": 0.5, "second weights": True, "opcode": "sub"},
        {"name": "f_bp", "from layer": "x", "to layer": "bp", "type": "fully connected", "plastic": False},
        {"name": "f_vc", "from layer": "x", "to layer": "v", "type": "convergent", "plastic": True,
         "convolutional": True, "arborized config": {"field size": 3, "wrap": True}},
        {"name": "f_spc", "from layer": "x", "to layer": "sp", "type": "convergent", "plastic": True,
         "convolutional": True, "connection variable": 2.0,
         "arborized config": {"field size": 3, "wrap": False}},
        {"name": "f_od", "from layer": "x", "to layer": "o", "type": "divergent", "plastic": True,
         "convolutional": True, "arborized config": {"field size": 2, "stride": 1, "wrap": False}},
        {"name": "p_q", "from layer": "out", "to layer": "q", "type": "one to one", "plastic": False},
        {"name": "p_r", "from layer": "v", "to layer": "r", "type": "one to one", "plastic": False},
        {"name": "p_z", "from layer": "h2", "to layer": "z", "type": "one to one", "plastic": False},
    ]}
    struct_conns = [c["name"] for c in net["connections"]]

    def inj_structs(rng, sizes):
        d = {("matrix", n, "weights"): rng.uniform(-0.5, 0.5, sizes["conn:" + n]).astype(np.float32)
             for n in struct_conns}
        d[("neuron", "ff", "p", "expected")] = rng.uniform(-1.0, 1.0, 9).astype(np.float32)
        return d
    out.append(Case("structures", net, 20, 141, inject=inj_structs,
                    inputs={"in": lambda rng, t, n: rng.normal(0.0, 1.0, n),
                            "x": lambda rng, t, n: rng.normal(0.0, 1.0, n),
                            "z": lambda rng, t, n: rng.normal(0.0, 1.0, n)},
                    record=[(st, l) for st, l in (("seq", "h1"), ("seq", "h2"), ("seq", "out"),
                                                  ("ff", "p"), ("ff", "o"), ("ff", "v"), ("ff", "sp"),
                                                  ("ff", "bp"), ("par", "q"), ("par", "r"), ("par", "z"))],
                    final=[("matrix", c, "weights") for c in ("f_p", "f_o", "f_v", "f_sp", "f_vc", "f_spc",
                                                              "f_od")]
                    + [("matrix", "f_sp", k) for k in ("var1", "var2")]
                    + [("neuron", "ff", "o", k) for k in ("state", "bold")]
                    + [("neuron", "ff", "bp", "error deltas"), ("neuron", "par", "z", "input"),
                       ("neuron", "ff", "sp", "input")]))
    return out


def _debug_case():
    """The debug model (a checker): every connection type into debug layers,
    plastic ones too, and a relay layer reading a debug layer.  Its layers'
    outputs stay zero and its neuron variable the dummy value."""
    net = {"structures": [{"name": "g", "type": "parallel", "layers": [
        _layer("src", "relay", 6, 8),
        _layer("d", "debug", 6, 8),
        _layer("e", "debug", 4, 5),
        _layer("out", "relay", 6, 8)]}],
        "connections": [
            {"name": "g_fc", "from layer": "src", "to layer": "e", "type": "fully connected",
             "plastic": True, "opcode": "add"},
            {"name": "g_sub", "from layer": "src", "to layer": "e", "type": "subset", "opcode": "add",
             "plastic": True,
             "subset config": {"from row start": 1, "from row end": 4, "from column start": 2,
                               "from column end": 6, "to row start": 0, "to row end": 2,
                               "to column start": 1, "to column end": 4}},
            {"name": "g_one", "from layer": "src", "to layer": "d", "type": "one to one",
             "plastic": False, "opcode": "add"},
            {"name": "g_conv", "from layer": "src", "to layer": "d", "type": "convergent",
             "plastic": True, "opcode": "add", "arborized config": {"field size": 3, "wrap": True}},
            {"name": "g_conv_clip", "from layer": "src", "to layer": "d", "type": "convergent",
             "plastic": False, "opcode": "add",
             "arborized config": {"field size": 3, "wrap": False}},
            {"name": "g_cnv", "from layer": "src", "to layer": "d", "type": "convergent",
             "convolutional": True, "plastic": True, "opcode": "add",
             "arborized config": {"field size": 3, "wrap": True}},
            {"name": "g_div", "from layer": "e", "to layer": "d", "type": "divergent",
             "plastic": True, "opcode": "add", "arborized config": {"field size": 3, "stride": 2}},
            {"name": "g_read", "from layer": "d", "to layer": "out", "type": "one to one",
             "plastic": False, "opcode": "add"}]}

    def inj(rng, sizes):
        return {("matrix", c, "weights"): rng.uniform(-1, 1, sizes["conn:" + c]).astype(np.float32)
                for c in ("g_fc", "g_sub", "g_one", "g_conv", "g_conv_clip", "g_cnv", "g_div",
                          "g_read")}
    return Case("debug", net, 10, 151, inject=inj,
                inputs={"src": lambda rng, t, n: rng.normal(0.0, 1.0, n)},
                record=[("g", "d"), ("g", "e"), ("g", "out")],
                final=[("neuron", "g", l, k) for l in ("d", "e") for k in ("neuron_var", "input")]
                + [("neuron", "g", "out", "input")])


CASES = {c.name: c for c in cases() + [_debug_case()]}
