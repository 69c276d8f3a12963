"""CPU oracle for the synaptogenesis per-timestep cycle (TEST INFRASTRUCTURE).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, and only as the checker.  The product never imports it.

It restates, in Python plus the C file ``sg_oracle.c``:
  * the JSON network schema with the reference's defaults and quirks
    (network/connection_config.cpp:8-45, 112-134, 207-257;
    network/layer_config.cpp:11-33; network/connection.cpp:7-61),
  * the state each neural model allocates (state/attributes.cpp:16-37,
    state/impl/izhikevich_attributes.cpp:587-757), in the reference's host
    layout, under the reference's variable names,
  * the engine's step order for parallel, sequential and feedforward
    structures (engine/engine.cpp:226-315, engine/cluster/parallel_cluster.cpp:
    27-131, engine/cluster/sequential_cluster.cpp:10-116,
    engine/cluster/cluster_node.cpp:7-212, engine/instruction.cpp:3-30),
    dendritic trees and second-order nodes (network/dendritic_node.cpp),
  * sparse compaction and randomized projections
    (state/weight_matrix.cpp:253-651),
  * every neural model but debug (state/impl/*_attributes.cpp).
Random initialisers of the reference are unseedable (util/tools.h:8); the
oracle draws them from a seeded numpy generator instead, and parity runs
inject every random quantity explicitly.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libsgoracle.so")

FLOAT, BIT, INT = 0, 1, 2
CONN_TYPES = {"fully connected": 0, "subset": 1, "one to one": 2, "convergent": 3, "divergent": 4}
OPCODES = {"add": 0, "sub": 1, "mult": 2, "div": 3, "pool": 4, "reward": 5, "modulate": 6,
           "gap": 7, "add_heaviside": 8, "sub_heaviside": 9, "mult_heaviside": 10}
MODELS = {"izhikevich": BIT, "relay": FLOAT, "game_of_life": BIT, "rate_encoding": FLOAT,
          "binary threshold": FLOAT, "backprop_rate_encoding": FLOAT,
          "hebbian_rate_encoding": FLOAT, "perceptron": FLOAT, "sine generator": FLOAT,
          "poisson generator": BIT, "spnet": BIT, "oscillator": FLOAT, "som": FLOAT,
          "nvm": FLOAT, "nvm_heaviside": FLOAT, "nvm_compare": FLOAT, "vp_max": FLOAT,
          "sample": FLOAT, "debug": FLOAT}
GLOBAL_SEED = 0x5EED5EED     # the library's default sg_set_seed value
# Which sine the reference's sine generator evaluates: its unqualified
# sin(float) resolves to the C library's double sin (pinned by the fixture).
SINE_USES_SINF = False


def rng_bits(seed, stream, index):
    """SplitMix64 finaliser of seed * A + stream * B + index (the library's
    counter-based generator, counter_rng.h)."""
    m = (1 << 64) - 1
    z = (seed * 0x9E3779B97F4A7C15 + stream * 0xD1B54A32D192ED03 + index) & m
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
    return z ^ (z >> 31)


def rng_below(seed, stream, index, n):
    return (rng_bits(seed, stream, index) >> 32) % n


def _rng_bits_np(seed, stream, index):
    """rng_bits over an array of indices (uint64)."""
    m = (1 << 64) - 1
    z = (seed * 0x9E3779B97F4A7C15 + stream * 0xD1B54A32D192ED03) & m
    z = (np.uint64(z) + np.asarray(index, np.uint64))
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


RNG_NOISE, RNG_NOISE_RATE = 6, 7
F32 = np.float32


def rng_open01(seed, stream, index):
    """Uniform draws in (0, 1): (24 random bits + 1) times the float nearest
    1 / (2^24 + 1)."""
    bits = _rng_bits_np(seed, stream, index) >> np.uint64(40)
    return (bits + np.uint64(1)).astype(np.float32) * F32(1.0 / 16777217.0)


def noise_log(x):
    """log x for x in (0, 1], float32 step by step: x = m 2^e, m in
    [sqrt(1/2), sqrt(2)), log m = 2 atanh((m - 1) / (m + 1)) by its series to
    the ninth power."""
    x = np.asarray(x, np.float32)
    u = x.view(np.uint32)
    e = ((u >> np.uint32(23)) & np.uint32(0xFF)).astype(np.int32) - 127
    m = ((u & np.uint32(0x7FFFFF)) | np.uint32(0x3F800000)).view(np.float32)
    big = m > F32(1.41421354)
    m = np.where(big, m * F32(0.5), m).astype(np.float32)
    e = np.where(big, e + 1, e)
    s = (m - F32(1.0)) / (m + F32(1.0))
    z = s * s
    p = F32(0.222222224) * z + F32(0.285714298)
    p = p * z + F32(0.400000006)
    p = p * z + F32(0.666666687)
    p = p * z + F32(2.0)
    return s * p + e.astype(np.float32) * F32(0.693147182)


def noise_cospi(x):
    """cos(pi x) for x in [0, 2], float32: folded onto [0, 1/4], then the
    Taylor series of cos (to t^10) or sin (to t^9)."""
    x = np.asarray(x, np.float32)
    x = np.where(x > F32(1.0), F32(2.0) - x, x).astype(np.float32)
    neg = x > F32(0.5)
    x = np.where(neg, F32(1.0) - x, x).astype(np.float32)
    sign = np.where(neg, F32(-1.0), F32(1.0)).astype(np.float32)
    t = (F32(0.5) - x) * F32(3.14159274)
    z = t * t
    p = F32(2.75573188e-06) * z - F32(1.98412701e-04)
    p = p * z + F32(8.33333377e-03)
    p = p * z - F32(0.166666672)
    p = p * z + F32(1.0)
    r_sin = t * p
    t = x * F32(3.14159274)
    z = t * t
    p = F32(-2.75573188e-07) * z + F32(2.48015876e-05)
    p = p * z - F32(1.38888892e-03)
    p = p * z + F32(4.16666679e-02)
    p = p * z - F32(0.5)
    r_cos = p * z + F32(1.0)
    return sign * np.where(x > F32(0.25), r_sin, r_cos).astype(np.float32)


def noise_draw(kind, seed, step, n, a, b, rates=None):
    """One step of init-config noise for n neurons (the library's k_noise):
    kind "uniform" (min a, max b), "normal" (mean a, std b), "poisson"
    (probability a or per-neuron rates; value b, returned as a mask and b)."""
    idx = (np.uint64(step) << np.uint64(32)) | np.arange(n, dtype=np.uint64)
    u = rng_open01(seed, RNG_NOISE * 4, idx)
    a, b = F32(a), F32(b)
    if kind == "uniform":
        return u * (b - a) + a
    if kind == "normal":
        u2 = rng_open01(seed, RNG_NOISE * 4 + 1, idx)
        normal = np.sqrt(F32(-2.0) * noise_log(u)) * noise_cospi(F32(2.0) * u2)
        return normal * b + a
    prob = rates if rates is not None else a
    return u < prob


def rng_uniform(seed, stream, index):
    """Counter-based uniform draw in [0, 1) (SplitMix64 finaliser of a
    linear mix of seed, stream and index), as the library's generators use."""
    m = (1 << 64) - 1
    z = (seed * 0x9E3779B97F4A7C15 + stream * 0xD1B54A32D192ED03) & m
    z = (np.uint64(z) + np.asarray(index, np.uint64))
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(40)).astype(np.float32) * np.float32(1.0 / 16777216.0)
IZ_PARAMS = {  # izhikevich_attributes.cpp:28-35
    "default": (0.02, 0.2, -70.0, 2), "regular": (0.02, 0.2, -65.0, 8),
    "bursting": (0.02, 0.2, -55.0, 4), "chattering": (0.02, 0.2, -50.0, 2),
    "fast": (0.1, 0.2, -65.0, 2), "low_threshold": (0.02, 0.25, -65.0, 2),
    "thalamo_cortical": (0.02, 0.25, -65.0, 0.05), "resonator": (0.1, 0.26, -65.0, 2)}


def build_lib():
    os.makedirs(_BUILD, exist_ok=True)
    src = os.path.join(HERE, "sg_oracle.c")
    if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                        "-o", _LIB_PATH, src, "-lm"], check=True)
    return _LIB_PATH


class _Conn(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in (
        "type", "opcode", "convolutional", "num_weights",
        "from_rows", "from_cols", "to_rows", "to_cols",
        "row_field", "col_field", "row_stride", "col_stride",
        "row_spacing", "col_spacing", "row_offset", "col_offset", "wrap",
        "fr0", "fr1", "fc0", "fc1", "tr0", "tr1", "tc0", "tc1")]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build_lib())
        _lib.sg_visits.restype = ctypes.c_long
        _lib.sg_istdp_src.restype = ctypes.c_float
        _lib.sg_istdp_dst.restype = ctypes.c_float
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


# ---------------------------------------------------------------------------
# Property semantics: values are strings (builder.cpp:15-39); the Python
# front-end converts bool -> "true"/"false" and everything else with str().
# ---------------------------------------------------------------------------
class Props:
    def __init__(self, d):
        self.d = {}
        self.children = {}
        self.arrays = {}
        self.child_arrays = {}
        for k, v in (d or {}).items():
            if v is None:
                continue
            if isinstance(v, dict):
                self.children[k] = Props(v)
            elif isinstance(v, list):
                for x in v:
                    if isinstance(x, dict):
                        self.child_arrays.setdefault(k, []).append(Props(x))
                    else:
                        self.arrays.setdefault(k, []).append(
                            ("true" if x else "false") if isinstance(x, bool) else str(x))
            else:
                self.d[k] = ("true" if v else "false") if isinstance(v, bool) else str(v)

    def has(self, k):
        return k in self.d

    def get(self, k, default=""):
        return self.d.get(k, default)

    def get_int(self, k, default):  # std::stoi: leading integer
        if k not in self.d:
            return default
        s = self.d[k].strip()
        i = 0
        if i < len(s) and s[i] in "+-":
            i += 1
        while i < len(s) and s[i].isdigit():
            i += 1
        return int(s[:i])

    def get_float(self, k, default):
        return float(np.float32(float(self.d[k]))) if k in self.d else float(np.float32(default))

    def get_bool(self, k, default):
        return self.d[k] == "true" if k in self.d else default

    def child(self, k):
        return self.children.get(k)


class Layer:
    def __init__(self, structure, p):
        self.structure = structure
        self.p = p
        self.name = p.get("name")
        self.model = p.get("neural model")
        if self.model not in MODELS:
            raise ValueError("oracle: unsupported neural model " + self.model)
        self.rows = p.get_int("rows", 0)
        self.cols = p.get_int("columns", 0)
        if self.rows <= 0 or self.cols <= 0:
            raise ValueError("invalid layer dimensions")
        self.size = self.rows * self.cols
        self.output_type = MODELS[self.model]
        self.inputs, self.outputs = [], []
        self.root = Dendrite("root", self, None, 0, OPCODES["add"], False, 0.0)
        self._add_dendrites(self.root, p.child_arrays.get("dendrites", []))
        self.registers = self.root.max_register() + 1

    def dendrites(self):  # breadth first, root first (layer.cpp:62-77)
        out = [self.root]
        for d in out:
            out.extend(ch for ch in d.children if isinstance(ch, Dendrite))
        return out

    def dendrite(self, name):
        for d in self.dendrites():
            if d.name == name:
                return d
        return None

    def _add_dendrites(self, parent, configs):  # layer.cpp:135-153, dendritic_node.cpp:80-104
        for dp in configs:
            if not dp.has("name"):
                raise ValueError("Attempted to dendrite without name to layer!")
            name = dp.get("name")
            if parent.second_order:
                raise ValueError("Second order dendritic nodes cannot have internal children!")
            if self.dendrite(name) is not None:
                raise ValueError("Duplicate dendritic node name: " + name + "!")
            node = Dendrite(name, self, parent, self.root.max_register() + 1,
                            OPCODES[dp.get("opcode", "add")], dp.get_bool("second order", False),
                            dp.get_float("init", 0.0))
            parent.children.append(node)
            self._add_dendrites(node, dp.child_arrays.get("children", []))


class Dendrite:
    """A node of a layer's dendritic tree (network/dendritic_node.cpp:5-52).
    children: internal Dendrite nodes and leaf Conn objects in creation
    order; a second-order node's first connection is its host (not a child)."""

    def __init__(self, name, layer, parent, reg, opcode, second_order, init):
        self.name, self.layer, self.parent, self.reg = name, layer, parent, reg
        self.opcode, self.second_order = opcode, second_order
        self.init = np.float32(init)
        self.children = []
        self.host = None

    def max_register(self):  # dendritic_node.cpp:142-153
        regs = [self.reg] + [ch.max_register() for ch in self.children if isinstance(ch, Dendrite)]
        return max(regs)


class Conn:
    def __init__(self, p, frm, to):
        self.p = p
        self.name = p.get("name", "")
        self.frm, self.to = frm, to
        self.plastic = p.get_bool("plastic", True)            # connection_config.cpp:213
        self.recurrent = p.get_bool("recurrent", False)
        self.delay = p.get_int("delay", 0)
        self.max_weight = p.get_float("max weight", 1.0)
        self.type = CONN_TYPES[p.get("type", "fully connected")]
        self.opcode = OPCODES[p.get("opcode", "add")]
        self.convolutional = p.get_bool("convolutional", False)
        # dendritic node and second-order role (connection.cpp:132-144)
        self.node = to.dendrite(p.get("dendrite", "root"))
        if self.node is None:
            raise ValueError("Cannot find Dendritic Node " + p.get("dendrite", "root") + "!")
        self.second_order = self.node.second_order
        self.so_host = self.second_order and self.node.host is None
        self.so_slave = self.second_order and not self.so_host
        self.sparse = p.get_bool("sparse", False) or p.get_bool("randomized projection", False)
        self.randomized = p.get_bool("randomized projection", False)
        if self.sparse and self.second_order:
            raise ValueError("Sparse second order connections are not supported!")
        if self.randomized and (self.convolutional or self.type in (0, 1)):
            raise ValueError("Cannot randomize projection on this weight matrix!")
        c = _Conn()
        c.type, c.opcode, c.convolutional = self.type, self.opcode, int(self.convolutional)
        c.from_rows, c.from_cols, c.to_rows, c.to_cols = frm.rows, frm.cols, to.rows, to.cols
        if self.type in (3, 4):
            a = p.child("arborized config")
            rf = a.get_int("row field size", 0)
            cf = a.get_int("column field size", 0)
            rs = a.get_int("row stride", 1)
            cs = a.get_int("column stride", 1)
            rsp = a.get_int("row spacing", 1)
            csp = a.get_int("column spacing", 1)
            ro = a.get_int("row offset", 0)
            co = a.get_int("row offset", 0)      # quirk: connection_config.cpp:16
            wrap = a.get_bool("wrap", False)
            if a.has("field size"):
                rf = cf = a.get_int("field size", 0)
            if a.has("stride"):
                rs = cs = a.get_int("stride", 0)
            if a.has("spacing"):
                rsp = csp = a.get_int("spacing", 0)
            if a.has("offset"):
                ro = co = a.get_int("offset", 0)
            if rf <= 0 or cf <= 0 or rs < 0 or cs < 0 or rsp < 1 or csp < 1:
                raise ValueError("invalid arborized config")
            if not a.has("row offset") and not a.has("offset"):
                ro = int(-rf / 2)
            if not a.has("column offset") and not a.has("offset"):
                co = int(-cf / 2)
            if self.type == 4 and (rs == 0 or cs == 0):
                raise ValueError("divergent connections cannot have zero stride")
            (c.row_field, c.col_field, c.row_stride, c.col_stride, c.row_spacing,
             c.col_spacing, c.row_offset, c.col_offset, c.wrap) = rf, cf, rs, cs, rsp, csp, ro, co, int(wrap)
            self.num_weights = rf * cf if self.convolutional else to.size * rf * cf
        elif self.type == 1:
            s = p.child("subset config")
            c.fr0, c.fr1 = s.get_int("from row start", 0), s.get_int("from row end", 0)
            c.tr0, c.tr1 = s.get_int("to row start", 0), s.get_int("to row end", 0)
            c.fc0, c.fc1 = s.get_int("from column start", 0), s.get_int("from column end", 0)
            c.tc0, c.tc1 = s.get_int("to column start", 0), s.get_int("to column end", 0)
            self.num_weights = (c.fr1 - c.fr0) * (c.fc1 - c.fc0) * (c.tr1 - c.tr0) * (c.tc1 - c.tc0)
        elif self.type == 2:
            if frm.rows != to.rows or frm.cols != to.cols:
                raise ValueError("one to one between differently sized layers")
            self.num_weights = to.size
        else:
            self.num_weights = frm.size * to.size
        c.num_weights = self.num_weights
        self.dense_num_weights = self.num_weights
        self.c = c
        if self.second_order and self.plastic:  # connection.cpp:149-153
            raise ValueError("Plastic second order connections are not supported!")
        if self.so_slave:  # connection.cpp:163-191
            host = self.node.host
            if (self.type != host.type or self.convolutional != host.convolutional
                    or self.num_weights != host.num_weights):
                raise ValueError("Second order connection does not match host connection!")
            if self.convolutional and (c.row_field * c.col_field != frm.size or c.row_spacing != 1
                                       or c.col_spacing != 1 or c.row_stride != 0 or c.col_stride != 0):
                raise ValueError("Second order convolutional connections must have fields that are "
                                 "the size of the input layer, and must have 0 stride and 1 spacing!")
        self._visits()

    def _visits(self):
        L = lib()
        rows = ctypes.c_int()
        n = L.sg_visits(ctypes.byref(self.c), ctypes.byref(rows), None, None, None, None, None, None)
        nrows = max(self.to.size, 1) + 1
        self.dst = np.zeros(nrows, np.int32)
        self.ptr = np.zeros(nrows + 1, np.int64)
        self.from_idx = np.zeros(max(n, 1), np.int32)
        self.w_idx = np.zeros(max(n, 1), np.int32)
        self.pre_row = np.zeros(max(n, 1), np.int32)
        self.pre_col = np.zeros(max(n, 1), np.int32)
        L.sg_visits(ctypes.byref(self.c), ctypes.byref(rows), _p(self.dst), _p(self.ptr),
                    _p(self.from_idx), _p(self.w_idx), _p(self.pre_row), _p(self.pre_col))
        self.rows = rows.value
        self.nvisits = n

    def _randomized_divergent(self, seed, n):
        """weight_matrix.cpp:443-504: the inverted convergent connection
        (layers swapped, same arborized config) randomized -- each source's
        window shifted so its first position is a random destination, indexed
        with the destination layer's row count as the row pitch -- and
        adjusted (wrapped or clipped), then every kept pair flipped into the
        divergent matrix at the destination's next free position."""
        c = self.c
        S, D = self.frm, self.to
        K = c.row_field * c.col_field
        fr = np.full(n, -1, np.int64)
        fc = np.full(n, -1, np.int64)
        fi = np.full(n, -1, np.int64)
        tr = np.full(n, -1, np.int64)
        tc = np.full(n, -1, np.int64)
        used = np.zeros(n, bool)
        count = np.zeros(D.size, np.int64)
        for s in range(S.size):
            sr, sc = divmod(s, S.cols)
            r0 = sr * c.row_stride + c.row_spacing * c.row_offset
            c0 = sc * c.col_stride + c.col_spacing * c.col_offset
            nr = rng_below(seed, 2 * s, 0, D.rows)
            nc = rng_below(seed, 2 * s + 1, 0, D.cols)
            for kr in range(c.row_field):
                for kc in range(c.col_field):
                    r = nr + kr * c.row_spacing
                    q = nc + kc * c.col_spacing
                    idx = r * D.rows + q
                    if c.wrap:
                        r, q = r % D.rows, q % D.cols
                        idx = r * D.cols + q
                    elif r < 0 or r >= D.rows or q < 0 or q >= D.cols:
                        continue
                    if idx < 0 or idx >= D.size:
                        raise ValueError("randomized projection indexes outside the layer")
                    slot = count[idx]
                    count[idx] += 1
                    if slot >= K:
                        raise ValueError("randomized divergent projection: more than K sources")
                    j = idx * K + slot
                    fr[j], fc[j], fi[j], tr[j], tc[j], used[j] = sr, sc, s, r, q, True
        return fr, fc, fi, tr, tc, used

    def sparsify(self, w):
        """WeightMatrix::sparsify + adjust_sparse_indices (weight_matrix.cpp:
        510-651, 253-338): keeps each matrix row's nonzero synapses, in order,
        in a [to_size][kmax] matrix padded with zero weights and -1 indices.
        The connection becomes SPARSE (connection.cpp:219-222); returns the
        compacted weights."""
        if self.convolutional:
            raise ValueError("Cannot sparsify convolutional weight matrix!")
        rows, cols = self.matrix_rows_cols()
        n_dense = self.num_weights
        nv = self.nvisits
        wi = self.w_idx[:nv]
        dst_of_visit = np.repeat(self.dst[:self.rows], np.diff(self.ptr[:self.rows + 1]))
        fr = np.full(n_dense, -1, np.int64)
        fc = np.full(n_dense, -1, np.int64)
        tr = np.full(n_dense, -1, np.int64)
        tc = np.full(n_dense, -1, np.int64)
        used = np.zeros(n_dense, bool)
        fr[wi], fc[wi] = self.pre_row[:nv], self.pre_col[:nv]
        tr[wi], tc[wi] = dst_of_visit // self.to.cols, dst_of_visit % self.to.cols
        used[wi] = True
        fi = np.where(used, fr * self.frm.cols + fc, -1)
        wc = self.p.child("weight config")
        seed = int(wc.get("seed")) if (wc is not None and wc.has("seed")) else \
            GLOBAL_SEED ^ ((0xA11CE5 * (self.index + 1)) & ((1 << 64) - 1))
        if self.randomized and self.type == 4:
            fr, fc, fi, tr, tc, used = self._randomized_divergent(seed, n_dense)
        elif self.randomized:   # weight_matrix.cpp:377-437, seeded draws
            for d in range(self.to.size):
                nr = rng_below(seed, 2 * d, 0, self.frm.rows)
                nc = rng_below(seed, 2 * d + 1, 0, self.frm.cols)
                if self.type == 2:
                    fr[d], fc[d], fi[d] = nr, nc, nr * self.frm.cols + nc
                else:
                    corner = d * cols
                    dr, dc = nr - fr[corner], nc - fc[corner]
                    fr[corner:corner + cols] += dr
                    fc[corner:corner + cols] += dc
                    fi[corner:corner + cols] = fr[corner:corner + cols] * self.frm.rows + fc[corner:corner + cols]
        visited = used.copy()
        used &= (w != 0.0)
        counts = used.reshape(rows, cols).sum(1)
        kmax = int(counts.max()) if rows else 0
        if kmax == 0:   # all-zero matrix: one synapse per row, where it exists
            kmax = 1
            first = np.arange(rows) * cols
            used[first] = visited[first]
        to_size = self.to.size
        n = kmax * to_size
        nw = np.zeros(n, np.float32)
        self.sp_from_row = np.full(n, -1, np.int64)
        self.sp_from_col = np.full(n, -1, np.int64)
        self.sp_to_row = np.full(n, -1, np.int64)
        self.sp_to_col = np.full(n, -1, np.int64)
        nonzero = np.zeros(to_size, np.int64)
        sp_fi = np.full(n, -1, np.int64)
        for r in range(rows):
            keep = np.nonzero(used[r * cols:(r + 1) * cols])[0] + r * cols
            j = r * kmax + np.arange(keep.size)
            nw[j] = w[keep]
            self.sp_from_row[j], self.sp_from_col[j] = fr[keep], fc[keep]
            self.sp_to_row[j], self.sp_to_col[j] = tr[keep], tc[keep]
            sp_fi[j] = fi[keep]
            nonzero[r] = keep.size
        # adjust_sparse_indices (weight_matrix.cpp:253-338): wrap and recompute,
        # or drop sources outside the layer and move the row's later sources
        # up (only the sources: weights and delays stay in place)
        wrap = self.type in (3, 4) and bool(self.c.wrap)
        frm_rows, frm_cols = self.frm.rows, self.frm.cols
        src = np.full(n, -1, np.int64)
        for r in range(to_size):
            kept = 0
            for k in range(nonzero[r]):
                j = r * kmax + k
                a, b, idx = self.sp_from_row[j], self.sp_from_col[j], sp_fi[j]
                if wrap:
                    a, b = a % frm_rows, b % frm_cols
                    idx = a * frm_cols + b
                elif a < 0 or a >= frm_rows or b < 0 or b >= frm_cols:
                    continue
                if idx < 0 or idx >= self.frm.size:
                    raise ValueError("randomized projection indexes outside the source layer")
                src[r * kmax + kept] = idx
                kept += 1
            nonzero[r] = kept
        # the kernel's view (synapse_kernel.h:303-366): row to of the compacted
        # matrix serves destination to (a subset's window rows land on the
        # layer's first destinations, as in the reference)
        self.type = 5
        self.num_weights = n
        self.kmax = kmax
        self.rows = to_size
        self.dst = np.arange(to_size + 1, dtype=np.int32)
        self.ptr = np.zeros(to_size + 2, np.int64)
        self.ptr[1:to_size + 1] = np.cumsum(nonzero)
        idx = np.concatenate([t * kmax + np.arange(nonzero[t]) for t in range(to_size)] or [np.zeros(0, int)])
        self.nvisits = idx.size
        self.w_idx = np.ascontiguousarray(np.append(idx, 0).astype(np.int32))
        self.from_idx = np.ascontiguousarray(np.append(src[idx], 0).astype(np.int32))
        self.pre_row = np.ascontiguousarray(np.append(self.sp_from_row[idx], 0).astype(np.int32))
        self.pre_col = np.ascontiguousarray(np.append(self.sp_from_col[idx], 0).astype(np.int32))
        return nw

    def matrix_rows_cols(self):  # connection.cpp:229-248
        if self.convolutional:
            rows = 1
        elif self.type == 1:
            rows = (self.c.tr1 - self.c.tr0) * (self.c.tc1 - self.c.tc0)
        else:
            rows = self.to.size
        if self.type == 1:
            cols = (self.c.fr1 - self.c.fr0) * (self.c.fc1 - self.c.fc0)
        elif self.type in (3, 4):
            cols = self.c.row_field * self.c.col_field
        elif self.type == 2:
            cols = 1
        else:
            cols = self.frm.size
        return rows, cols


class OracleNetwork:
    """Builds the network and its state from a reference-schema dict."""

    def __init__(self, net, seed=0, weight_callbacks=None):
        """weight_callbacks: {name: fn(id, weights)} for weight configs with a
        "callback" (weight_matrix.cpp:853-869); fn fills the dense weights in
        place before any sparsification."""
        self.rng = np.random.default_rng(seed)
        self.weight_callbacks = weight_callbacks or {}
        top = Props(net)
        self.layers, self.conns, self.structures = [], [], []
        self.cluster_type = {}
        for sp in top.child_arrays.get("structures", []):
            sname = sp.get("name")
            self.cluster_type[sname] = sp.get("type", "parallel")
            self.structures.append(sname)
            for lp in sp.child_arrays.get("layers", []):
                layer = Layer(sname, lp)
                layer.cluster_type = self.cluster_type[sname]
                self.layers.append(layer)
        for cp in top.child_arrays.get("connections", []):
            frm = self._find(cp.get("from layer"), cp.get("from structure", None))
            to = self._find(cp.get("to layer"), cp.get("to structure", None))
            conn = Conn(cp, frm, to)
            conn.index = len(self.conns)
            frm.outputs.append(conn)
            to.inputs.append(conn)
            if conn.so_host:  # dendritic_node.cpp:106-140
                conn.node.host = conn
            else:
                conn.node.children.append(conn)
            self.conns.append(conn)
        self.order = {st: self._order_structure(st) for st in self.structures
                      if self.cluster_type[st] != "parallel"}
        self._build_state()

    def _order_structure(self, st):
        """SequentialCluster / FeedforwardCluster (sequential_cluster.cpp:
        10-67, feedforward_cluster.cpp:8-36): layers placed backwards from the
        structure's outputs, each before the layers it feeds."""
        layers = [l for l in self.layers if l.structure == st]
        inner = lambda c: c.frm.structure == st and c.to.structure == st
        queue = [l for l in layers
                 if all(not (c.to.structure == st and not c.recurrent) for c in l.outputs) or not l.outputs]
        placed, stalled = [], 0
        while queue:
            cur = queue.pop(0)
            if cur in placed:
                stalled = 0
                continue
            if any(c.to is not cur and inner(c) and not c.recurrent and c.to not in placed
                   for c in cur.outputs):
                queue.append(cur)
                stalled += 1
                if stalled > len(queue):
                    break
                continue
            stalled = 0
            placed.append(cur)
            queue.extend(c.frm for c in cur.inputs
                         if c.frm is not cur and inner(c) and not c.recurrent and c.frm not in placed)
        if len(placed) < len(layers):
            raise ValueError("Sequential cluster failed to process all layers!")
        if self.cluster_type[st] == "feedforward":
            def acyclic(l, path):
                if l in path:
                    return False
                path.append(l)
                ok = all(acyclic(c.to, path) for c in l.outputs if c.to.structure == st)
                path.pop()
                return ok
            for l in layers:
                if all(not (c.frm.structure == st and not c.recurrent) for c in l.inputs) \
                        and not acyclic(l, []):
                    raise ValueError("Feedforward engine requires a structure with no cycles!")
        return placed[::-1]

    def _find(self, name, structure):
        hits = [l for l in self.layers if l.name == name and (structure is None or l.structure == structure)]
        if len(hits) != 1:
            raise ValueError("cannot resolve layer " + str(name))
        return hits[0]

    # -- state ------------------------------------------------------------
    def _build_state(self):
        self.neuron = {}
        self.matrix = {}
        self.so_weights = {}
        L = lib()
        for l in self.layers:
            max_delay = max([c.delay for c in l.outputs] + [0])
            l.history = 1 + (max_delay // 32 if l.output_type == BIT else max_delay)
            st = {"input": np.zeros(l.registers * l.size, np.float32),   # attributes.cpp:21-26
                  "output": np.zeros(l.history * l.size, np.uint32)}
            if l.model in ("backprop_rate_encoding", "sample") and l.cluster_type != "feedforward":
                raise ValueError("Cluster compatibility conflict detected!")   # feedforward only
            if l.model == "backprop_rate_encoding":
                st["error deltas"] = np.zeros(l.size, np.float32)
            if l.model == "sample":
                st["neuron_var"] = np.zeros(l.size, np.float32)
            elif l.model == "debug":   # debug_attributes.cpp:140-146: DUMMY_VAL
                st["neuron_var"] = np.ones(l.size, np.float32)
            elif l.model == "perceptron":
                st["expected"] = np.zeros(l.size, np.float32)
            elif l.model == "oscillator":   # oscillator_attributes.cpp:12-22
                st["state"] = np.zeros(l.size, np.float32)
                st["bold"] = np.zeros(l.size, np.float32)
            elif l.model.startswith("nvm"):   # nvm_attributes.cpp:12-27
                off = np.float32(1.0 - float(np.float32(l.p.get("noise offset", "0.5"))))
                if off > 1.0 or off < 0.0:
                    raise ValueError("Noise offset must be in [0,1]!")
                st["state"] = np.zeros(l.size, np.float32)
                st["context"] = np.ones(l.size, np.float32)
                if l.model == "nvm_compare":
                    st["true_state"] = np.zeros(l.size, np.float32)
                    l.tolerance = np.float32(1.0 - float(np.float32(l.p.get("tolerance", "1.0"))))
                l.gates = np.array([1.0, 0.0, 0.0], np.float32)   # activity, learning, noise
                l.gain = np.float32(l.p.get("gain", "1."))
            elif l.model == "som":   # som_attributes.cpp:100-106
                st["plasticity"] = np.zeros(l.size, np.float32)
                l.winner = 0
            l.iteration = 0     # sine / Poisson generator step count
            if l.model == "spnet":   # spnet_attributes.cpp:369-425
                for k in ("voltage", "recovery", "post trace"):
                    st[k] = np.zeros(l.size, np.float32)
                st["time since spike"] = np.full(l.size, 32, np.int32)
                a, b, c, d = IZ_PARAMS[l.p.get("params", "regular")]
                for k, v in zip("abcd", (a, b, c, d)):
                    st[k] = np.full(l.size, v, np.float32)
                L.sg_iz_init(l.size, _p(st["a"]), _p(st["b"]), _p(st["c"]),
                             _p(st["voltage"]), _p(st["recovery"]))
            if l.model == "izhikevich":
                for k in ("ampa", "nmda", "gabaa", "gabab", "mult", "dopamine",
                          "voltage", "recovery", "post trace"):
                    st[k] = np.zeros(l.size, np.float32)
                st["time since spike"] = np.full(l.size, 32, np.int32)
                a, b, c, d = IZ_PARAMS[l.p.get("params", "regular")]
                for k, v in zip("abcd", (a, b, c, d)):
                    st[k] = np.full(l.size, v, np.float32)
                L.sg_iz_init(l.size, _p(st["a"]), _p(st["b"]), _p(st["c"]),
                             _p(st["voltage"]), _p(st["recovery"]))
            self.neuron[l] = st
        for c in self.conns:
            w = self._init_weights(c)
            if c.sparse:
                w = c.sparsify(w)
            self.matrix[c] = m = {"weights": w}
            if c.so_host:  # weight_matrix.cpp:79-80 (not readable through the getters)
                self.so_weights[c] = np.zeros(c.num_weights, np.float32)
            if c.to.model == "som":   # som_attributes.cpp:108-121
                m["output cache"] = np.zeros(c.num_weights, np.float32)
                c.learning_rate = c.p.get_float("learning rate", 0.01)
                c.neighbor_learning_rate = c.p.get_float("neighbor learning rate", 0.001)
                c.neighborhood_size = c.p.get_int("neighborhood size", 2)
            if c.to.model in ("som", "oscillator") and (c.second_order or
                                                        (c.to.model == "som" and c.convolutional)):
                raise ValueError("Unimplemented connection type!")
            if c.to.model == "sample":   # sample_attributes.cpp:22-45
                if c.second_order:
                    raise ValueError("Unimplemented connection type!")
                m["var1"] = np.zeros(c.num_weights, np.float32)
                m["var2"] = np.zeros(c.num_weights, np.float32)
                if c.p.get("second weights", "false") == "true":
                    val = c.frm.p.get_float("value", 1.0)
                    if val < 0:
                        raise ValueError("Val cannot be negative!")
                    m["var1"][:] = m["weights"] * np.float32(val)
                if c.opcode == OPCODES["sub"]:
                    m["var2"][:] = 1.0
            if c.to.model == "spnet":   # spnet_attributes.cpp:440-494
                n = c.num_weights
                m["presyn trace"] = np.zeros(n, np.float32)
                m["time since spike"] = np.full(n, 32, np.int32)
                m["weight derivative"] = np.zeros(n, np.float32)
                m["delays"] = self._default_delays(c)
                c.baseline_conductance = c.p.get_float("conductance", 1.0)
                c.learning_rate = c.p.get_float("learning rate", 0.1)
            if c.to.model == "izhikevich":
                n = c.num_weights
                m["short trace"] = np.zeros(n, np.float32)
                m["long trace"] = np.zeros(n, np.float32)
                m["presyn trace"] = np.zeros(n, np.float32)
                m["short term R"] = np.ones(n, np.float32)
                # quirk F4: compares the ConnectionType with the ADD/SUB opcodes
                # (izhikevich_attributes.cpp:723-728)
                m["short term w"] = np.full(n, 0.5 if c.type == 0 else (0.2 if c.type == 1 else 0.0),
                                            np.float32)
                m["weight derivatives"] = np.full(n, 0.000001, np.float32)
                m["time since spike"] = np.full(n, 32, np.int32)
                if "delays" not in m:
                    m["delays"] = self._default_delays(c)
                c.baseline_conductance = c.p.get_float("conductance", 1.0)
                c.learning_rate = c.p.get_float("learning rate", 0.1)
                c.stp_flag = c.p.get("short term plasticity", "true") == "true"

    def _init_weights(self, c):
        wc = c.p.child("weight config") or Props({})
        n = c.num_weights
        t = wc.get("type", "flat")
        if t == "flat":
            w = np.full(n, wc.get_float("weight", 1.0), np.float32)
            frac = wc.get_float("fraction", 1.0)
            if frac != 1.0:
                w = np.where(self.rng.random(n) < frac, w, 0).astype(np.float32)
        elif t == "random":
            w = self.rng.uniform(wc.get_float("min weight", 0.0),
                                 wc.get_float("max weight", c.max_weight), n).astype(np.float32)
        elif t == "specified":
            vals = [float(x) for x in wc.get("weight string").split()]
            w = np.array(vals[:n], np.float32)
        else:
            raise ValueError("oracle: weight config " + t)
        if wc.has("callback"):
            self.weight_callbacks[wc.get("callback")](wc.get_int("id", 0), w)
        if not wc.get_bool("diagonal", True):   # weight_matrix.cpp:951-977
            if c.type == 0:
                w[np.arange(c.frm.size) * c.frm.size + np.arange(c.frm.size)] = 0
            elif c.type == 1:
                fs = (c.c.fr1 - c.c.fr0) * (c.c.fc1 - c.c.fc0)
                w[np.arange(fs) * fs + np.arange(fs)] = 0
            elif c.type == 3:
                self._circular_mask(c, w, radius=0.5, invert=True, value=0.0)
        return w

    @staticmethod
    def _circular_mask(c, w, radius, invert, value):  # weight_matrix.cpp:749-824
        rf, cf = c.c.row_field, c.c.col_field
        rr = cr = np.float32(radius)
        rc, cc = np.float32(rf) / np.float32(2), np.float32(cf) / np.float32(2)
        rsq, csq = np.float32(rr * rr), np.float32(cr * cr)
        sq_mult = np.float32(rsq * csq)
        K = rf * cf
        reps = 1 if c.convolutional else c.to.size
        for kr in range(rf):
            for kc in range(cf):
                a = np.float32(np.float64(kr) + 0.5 - np.float64(rc))
                b = np.float32(np.float64(kc) + 0.5 - np.float64(cc))
                term = np.float32(np.float32(a * a) * csq) + np.float32(np.float32(b * b) * rsq)
                if invert == (term <= sq_mult):
                    w[np.arange(reps) * K + kr * cf + kc] = value

    def _default_delays(self, c):  # izhikevich_attributes.cpp:732-751
        n = c.num_weights
        if c.p.get("myelinated", "false") == "true":
            return np.full(n, c.delay, np.int32)
        if c.p.has("random delay"):
            raise ValueError("oracle: 'random delay' crashes the reference (unallocated delays)")
        fr = np.full(n, -1, np.int32)
        fcol = np.full(n, -1, np.int32)
        tr = np.full(n, -1, np.int32)
        tcol = np.full(n, -1, np.int32)
        dst_of_visit = np.repeat(c.dst[:c.rows], np.diff(c.ptr[:c.rows + 1]))
        wi = c.w_idx[:c.nvisits]
        fr[wi] = c.pre_row[:c.nvisits]
        fcol[wi] = c.pre_col[:c.nvisits]
        tr[wi] = dst_of_visit // c.to.cols
        tcol[wi] = dst_of_visit % c.to.cols
        if c.type == 5:   # compacted indices, before wrapping, -1 pads
            fr, fcol = c.sp_from_row.astype(np.int32), c.sp_from_col.astype(np.int32)
            tr, tcol = c.sp_to_row.astype(np.int32), c.sp_to_col.astype(np.int32)
        dist = np.zeros(n, np.float32)
        delays = np.zeros(n, np.int32)
        rc = lib().sg_distance_delays(
            ctypes.c_long(n), _p(fr), _p(fcol), _p(tr), _p(tcol),
            ctypes.c_float(c.frm.p.get_float("neuron spacing", 0.1)),
            ctypes.c_float(c.to.p.get_float("neuron spacing", 0.1)),
            ctypes.c_float(c.p.get_float("x offset", 0.0)),
            ctypes.c_float(c.p.get_float("y offset", 0.0)),
            ctypes.c_float(0.15), int(c.p.get("cap delay", "false") == "true"),
            c.delay, _p(dist), _p(delays))
        if rc != 0:
            raise ValueError("BIT delays cannot be greater than 31")
        return delays

    # -- init-config noise (instruction.h:200-282, kernel.cpp:42-158) --------
    def _noise_seed(self, l):
        init = l.p.child("init config")
        if init.has("seed"):
            return int(init.get("seed"))
        return (GLOBAL_SEED ^ (0xA5A5 * (self.layers.index(l) + 1))) & ((1 << 64) - 1)

    def _noise(self, l, init, kind, reg0, is_input):
        """The layer's noise of this step, drawn like the library's
        counter-based generator from (seed, the layer's step, neuron);
        overwrites a layer without input, adds onto an input layer's."""
        if not hasattr(self, "noise_step"):
            self.noise_step = {}
        t = self.noise_step.get(l.name, 0)
        seed = self._noise_seed(l)
        if kind == "uniform":
            v = noise_draw(kind, seed, t, l.size, init.get_float("min", 0.0),
                           init.get_float("max", 1.0))
        elif kind == "normal":
            v = noise_draw(kind, seed, t, l.size, init.get_float("mean", 1.0),
                           init.get_float("std dev", 0.1))
        else:
            rate = np.float32(0.001) * np.float32(init.get_float("rate", 1.0))
            rates = None
            if init.get("random", "false") == "true":
                rates = rng_uniform(seed, RNG_NOISE_RATE, np.arange(l.size)) * rate
            fire = noise_draw(kind, seed, t, l.size, rate, 0.0, rates)
            value = np.float32(init.get_float("value", 20.0))
            if is_input:
                reg0[fire] += value
            else:
                reg0[:] = np.where(fire, value, np.float32(0.0))
            self.noise_step[l.name] = t + 1
            return
        if is_input:
            reg0 += v
        else:
            reg0[:] = v
        self.noise_step[l.name] = t + 1

    # -- accessors mirroring the reference's getters -------------------------
    def layer(self, name):
        return self._find(name, None)

    def connection(self, name):
        hits = [c for c in self.conns if c.name == name]
        return hits[-1]

    def get_neuron_data(self, layer, key):
        return self.neuron[self.layer(layer)][key]

    def get_weight_matrix(self, conn, key="weights"):
        return self.matrix[self.connection(conn)][key]

    # -- engine build ------------------------------------------------------
    def start_engine(self):
        """What building an engine does to the state: internal dendritic
        registers other than second-order ones are set to their init values
        (cluster_node.cpp:116-129).  run() calls it; step() calls it once."""
        for l in self.layers:
            for d in l.dendrites():
                if d is not l.root and not d.second_order:
                    self.neuron[l]["input"][d.reg * l.size:(d.reg + 1) * l.size] = d.init
        self._engine_started = True

    def _dendrite_plan(self, node, ops):  # cluster_node.cpp:115-207 (post-order)
        if node.second_order:
            ops.append(("copy", node))
        for ch in node.children:
            if isinstance(ch, Dendrite):
                self._dendrite_plan(ch, ops)
                if node.reg != ch.reg:
                    ops.append(("fold", node, ch))
            else:
                ops.append(("conn", ch, node))
        if node.second_order:
            if node.host is None:
                raise ValueError("Missing host connection for second order node!")
            ops.append(("conn", node.host, node))
        return ops

    # -- one timestep ------------------------------------------------------
    def step(self, inputs=None, learning=True):
        """inputs: {layer name: float32 array} for layers fed by an input module."""
        if not getattr(self, "_engine_started", False):
            self.start_engine()
        inputs = inputs or {}
        L = lib()
        # init / input transfer into register 0 (instruction.cpp:3-30,
        # instruction.h:474-489), and the models' init keys
        # (cluster_node.cpp:46-50)
        for l in self.layers:
            if l.model == "oscillator":
                self.neuron[l]["bold"][:] = 0.0
            reg0 = self.neuron[l]["input"][:l.size]
            init = l.p.child("init config")
            is_input = l.name in inputs
            if is_input:
                reg0[:] = np.asarray(inputs[l.name], np.float32)
            if init is not None:
                kind = init.get("type", "normal")
                if kind == "flat":
                    v = np.float32(init.get_float("value", 1.0))
                    if is_input:
                        reg0 += v
                    else:
                        reg0[:] = v
                elif kind in ("uniform", "normal", "poisson"):
                    self._noise(l, init, kind, reg0, is_input)
                else:
                    raise ValueError("Unrecognized init type: " + kind)
            elif not is_input:
                reg0[:] = 0.0
        if not self.order:
            # synaptic activation: every connection reads outputs of step t-1
            for l in self.layers:
                self._activate_layer(L, l)
            # neuron updates
            for l in self.layers:
                self._update(L, l)
        else:
            # the clusters' order (engine.cpp:226-315): parallel structures'
            # non-input layers activate before the input is read
            # (parallel_cluster.cpp:27-79, 105-118); then each structure in
            # turn, a sequential one updating each layer right after its
            # activations; then the parallel layers' updates
            for st in self.structures:
                if st not in self.order:
                    for l in self.layers:
                        if l.structure == st and l.name not in inputs:
                            self._activate_layer(L, l)
            for st in self.structures:
                if st not in self.order:
                    for l in self.layers:
                        if l.structure == st and l.name in inputs:
                            self._activate_layer(L, l)
                else:
                    for l in self.order[st]:
                        self._activate_layer(L, l)
                        self._update(L, l)
            for st in self.structures:
                if st not in self.order:
                    for l in self.layers:
                        if l.structure == st:
                            self._update(L, l)
        # plasticity
        if learning:
            for c in self.conns:
                bound = c.frm.structure == c.to.structure and c.to.cluster_type == "feedforward"
                if c.plastic and c.to.model in ("perceptron", "oscillator", "vp_max", "sample"):
                    if not bound:
                        raise ValueError(c.to.model + " learning reads source outputs that the "
                                         "reference binds only in feedforward structures")

            for l in self.layers:
                for c in l.inputs:
                    if c.plastic and c.to.model == "izhikevich":
                        self._learn(L, c)
                    elif c.plastic and c.to.model == "spnet":
                        self._learn_spnet(L, c)
                    elif c.plastic and c.to.model == "perceptron":   # perceptron_attributes.cpp:51-60
                        L.sg_upd_perceptron(c.rows, _p(c.dst), _p(c.ptr), _p(c.from_idx), _p(c.w_idx),
                                            _p(self._src_words(c)), _p(self.neuron[c.to]["output"]),
                                            _p(self.neuron[c.to]["expected"]), _p(self.matrix[c]["weights"]))
                    elif c.plastic and c.convolutional and c.to.model in ("oscillator", "vp_max",
                                                                          "sample"):
                        rate = c.p.get_float("connection variable", 1.0) if c.to.model == "sample" else 1.0
                        L.sg_upd_toward_post_conv(ctypes.byref(c.c), _p(self._src_words(c)),
                                                  c.frm.output_type, c.delay,
                                                  _p(self.neuron[c.to]["output"]), ctypes.c_float(rate),
                                                  _p(self.matrix[c]["weights"]))
                    elif c.plastic and c.to.model in ("oscillator", "vp_max"):
                        L.sg_upd_toward_post(c.rows, _p(c.dst), _p(c.ptr), _p(c.from_idx), _p(c.w_idx),
                                             _p(self._src_words(c)), c.frm.output_type, c.delay,
                                             _p(self.neuron[c.to]["output"]), ctypes.c_float(1.0),
                                             _p(self.matrix[c]["weights"]))
                    elif c.plastic and c.to.model == "sample":
                        # its updater is its activator (sample_attributes.cpp:229-247)
                        self._activate(L, c)
                    elif c.plastic and c.to.model == "som":   # som_attributes.cpp:58-79
                        m = self.matrix[c]
                        L.sg_upd_som(c.rows, _p(c.dst), _p(c.ptr), _p(c.w_idx), c.to.cols, c.to.winner,
                                     _p(self.neuron[c.to]["plasticity"]), _p(m["output cache"]),
                                     ctypes.c_float(c.learning_rate),
                                     ctypes.c_float(c.neighbor_learning_rate), c.neighborhood_size,
                                     _p(m["weights"]))

    def run(self, steps, input_fn=None, learning=True, record=None):
        """record: list of (layer, key) recorded after every step."""
        trace = {k: [] for k in (record or [])}
        self.start_engine()
        for t in range(steps):
            self.step(input_fn(t) if input_fn else None, learning)
            for k in trace:
                trace[k].append(self.neuron[self.layer(k[0])][k[1]].copy())
        return {k: np.stack(v) for k, v in trace.items()}

    def _src_words(self, c):
        out = self.neuron[c.frm]["output"]
        w = c.delay // 32 if c.frm.output_type == BIT else c.delay
        return out[w * c.frm.size:(w + 1) * c.frm.size]

    def _activate(self, L, c):
        if c.to.model == "debug":   # debug activators only check indices
            return
        st, m = self.neuron[c.to], self.matrix[c]
        src = self._src_words(c)
        geo = (c.rows, _p(c.dst), _p(c.ptr), _p(c.from_idx), _p(c.w_idx))
        reg = st["input"][c.node.reg * c.to.size:(c.node.reg + 1) * c.to.size]
        direct = c.p.get("direct", "false") == "true"
        if c.to.model == "izhikevich" and not direct and c.second_order:
            raise ValueError("Unimplemented connection type!")   # izhikevich_attributes.cpp:371-379
        if c.so_slave:
            so = self.so_weights[c.node.host]
            if c.convolutional:
                L.sg_act_second_order_conv(c.frm.size, _p(src), c.frm.output_type, c.delay, c.opcode,
                                           _p(m["weights"]), _p(so))
            else:
                L.sg_act_second_order(*geo, _p(src), c.frm.output_type, c.delay, c.opcode,
                                      _p(m["weights"]), _p(so))
            return
        if c.to.model == "spnet":   # spnet_attributes.cpp:202-214
            if c.second_order:
                raise ValueError("Unimplemented connection type!")
            L.sg_act_spnet(*geo, _p(src), c.frm.output_type, _p(m["weights"]), _p(m["delays"]),
                           _p(m["time since spike"]), ctypes.c_float(c.baseline_conductance),
                           c.opcode, _p(reg))
            return
        if c.to.model.startswith("nvm"):
            self._activate_nvm(L, c, st, m, src, geo, reg)
            return
        if c.to.model == "vp_max":   # vp_max_attributes.cpp:72-85
            if c.second_order:
                raise ValueError("Unimplemented connection type!")
            L.sg_act_vp_max(*geo, _p(src), c.frm.output_type, c.delay, c.opcode, _p(m["weights"]),
                            _p(reg))
            return
        if c.to.model == "oscillator":
            L.sg_act_oscillator(*geo, _p(src), c.frm.output_type, c.delay, c.opcode,
                                _p(m["weights"]), _p(reg), _p(st["bold"]))
            return
        if c.to.model == "som":
            L.sg_act_som(*geo, _p(src), c.frm.output_type, c.delay, int(c.opcode == OPCODES["modulate"]),
                         _p(m["weights"]), _p(m["output cache"]), _p(reg), _p(st["plasticity"]))
            return
        if c.to.model == "perceptron":   # perceptron_attributes.cpp:35-47
            if c.second_order or c.convolutional:
                raise ValueError("Unimplemented connection type!")
            L.sg_act_perceptron(*geo, _p(src), c.frm.output_type, c.delay, c.opcode,
                                _p(m["weights"]), _p(reg))
            return
        if c.to.model == "izhikevich" and not direct:
            if c.opcode == OPCODES["gap"]:
                L.sg_act_gap(*geo, _p(st["voltage"]), _p(m["weights"]), _p(reg))
                return
            targets = {0: ("ampa", 0.8, "nmda", 0.993), 1: ("gabaa", 0.833, "gabab", 0.993),
                       2: ("mult", 0.95, None, -1.0), 5: ("dopamine", 0.95, None, -1.0)}
            if c.opcode not in targets:
                raise ValueError("Unimplemented connection type!")
            sname, stau, lname, ltau = targets[c.opcode]
            L.sg_act_iz(*geo, _p(src), c.frm.output_type, _p(m["weights"]), _p(m["short term R"]),
                        _p(m["short term w"]), _p(m["delays"]), _p(m["time since spike"]),
                        _p(m["short trace"]), _p(m["long trace"]),
                        ctypes.c_float(c.baseline_conductance), ctypes.c_float(stau),
                        ctypes.c_float(ltau), _p(st[sname]), _p(st[lname] if lname else st[sname]))
        else:
            w = self.so_weights[c] if c.so_host else m["weights"]
            L.sg_act_base(*geo, _p(src), c.frm.output_type, c.delay, c.opcode, _p(w), _p(reg))

    def _activate_layer(self, L, l):
        if l.registers == 1:
            for c in l.inputs:
                self._activate(L, c)
            return
        inp = self.neuron[l]["input"]
        for op in self._dendrite_plan(l.root, []):
            if op[0] == "copy":  # instruction.h:461-472
                host = op[1].host
                self.so_weights[host][:] = self.matrix[host]["weights"]
            elif op[0] == "fold":
                node, ch = op[1], op[2]
                L.sg_calc_internal(l.size, _p(inp[ch.reg * l.size:]), _p(inp[node.reg * l.size:]),
                                   ch.opcode, ctypes.c_float(ch.init))
            else:
                self._activate(L, op[1])

    def _update(self, L, l):
        st = self.neuron[l]
        if l.model == "izhikevich":
            L.sg_iz_neurons(l.size, l.history, _p(st["input"]), _p(st["output"]),
                            *[_p(st[k]) for k in ("ampa", "nmda", "gabaa", "gabab", "mult",
                                                  "dopamine", "voltage", "recovery", "post trace",
                                                  "time since spike", "a", "b", "c", "d")])
        elif l.model == "relay":
            L.sg_relay(l.size, l.history, _p(st["input"]), _p(st["output"]),
                       int(l.p.get("ramp", "false") == "true"))
        elif l.model in ("rate_encoding", "backprop_rate_encoding", "hebbian_rate_encoding"):
            L.sg_rate(l.size, l.history, _p(st["input"]), _p(st["output"]))
        elif l.model == "spnet":
            L.sg_spnet_neurons(l.size, l.history, _p(st["input"]), _p(st["output"]),
                               *[_p(st[k]) for k in ("voltage", "recovery", "post trace",
                                                     "time since spike", "a", "b", "c", "d")])
        elif l.model.startswith("nvm"):
            if l.gates[2] != 0.0:
                raise ValueError("oracle: NVM noise draws are not restated")
            L.sg_nvm_update(int(l.model != "nvm"), l.size, l.history, _p(st["input"]), _p(st["state"]),
                            _p(st["context"]), _p(st["output"]), ctypes.c_float(l.gain))
        elif l.model == "oscillator":
            L.sg_oscillator(l.size, l.history, ctypes.c_float(l.p.get_float("tonic", 0.0)),
                            ctypes.c_float(l.p.get_float("tau", 0.1)),
                            ctypes.c_float(l.p.get_float("decay", 0.1)), _p(st["input"]),
                            _p(st["state"]), _p(st["bold"]), _p(st["output"]))
        elif l.model == "som":
            w = ctypes.c_int()
            L.sg_som(l.size, l.history, ctypes.c_float(l.p.get_float("rbf scale", 1.0)),
                     _p(st["input"]), _p(st["output"]), ctypes.byref(w))
            l.winner = w.value
        elif l.model == "vp_max":
            L.sg_relay(l.size, l.history, _p(st["input"]), _p(st["output"]), 0)
        elif l.model == "sample":   # sample_attributes.cpp:52-58: layer variable 0
            L.sg_scale(l.size, l.history, ctypes.c_float(0.0), _p(st["input"]), _p(st["output"]))
        elif l.model == "binary threshold":
            L.sg_bin_thresh(l.size, l.history, _p(st["input"]), _p(st["output"]))
        elif l.model == "perceptron":
            per_neuron = sum(c.num_weights for c in l.inputs) // l.size   # layer.cpp:110-115
            L.sg_perceptron(l.size, l.history, per_neuron, _p(st["input"]), _p(st["output"]))
        elif l.model == "sine generator":
            freq = np.float32(2 * np.pi / 1000 * np.float64(np.float32(l.p.get("frequency", "10"))))
            L.sg_sine(l.size, l.history, ctypes.c_float(freq), l.iteration, int(SINE_USES_SINF),
                      _p(st["input"]), _p(st["output"]))
            l.iteration += 1
        elif l.model == "poisson generator":
            seed = int(l.p.get("seed")) if l.p.has("seed") else \
                GLOBAL_SEED ^ ((0xC0FFEE1234567 * (self.layers.index(l) + 1)) & ((1 << 64) - 1))
            draws = rng_uniform(seed, l.iteration, np.arange(l.size))
            L.sg_poisson_gen(l.size, l.history, _p(draws), _p(st["input"]), _p(st["output"]))
            l.iteration += 1
        elif l.model == "game_of_life":
            L.sg_gol(l.size, l.history, _p(st["input"]), _p(st["output"]),
                     l.p.get_int("survival_min", 2), l.p.get_int("survival_max", 3),
                     l.p.get_int("birth_min", 3), l.p.get_int("birth_max", 3))

    def _learn(self, L, c):
        if c.convolutional:
            raise ValueError("Unimplemented connection type!")
        if c.opcode not in (0, 1):
            raise ValueError("Unimplemented connection type!")
        st, m, ft = self.neuron[c.to], self.matrix[c], self.matrix[c]["time since spike"]
        L.sg_upd_iz(c.rows, _p(c.dst), _p(c.ptr), _p(c.from_idx), _p(c.w_idx),
                    c.frm.output_type, int(c.opcode == 1), ctypes.c_float(c.learning_rate), int(c.stp_flag),
                    ctypes.c_float(c.max_weight), _p(st["post trace"]), _p(st["time since spike"]),
                    _p(st["output"][:c.to.size]), _p(ft), _p(m["weights"]), _p(m["presyn trace"]),
                    _p(m["weight derivatives"]), _p(m["short term R"]), _p(m["short term w"]))

    def _learn_spnet(self, L, c):  # spnet_attributes.cpp:288-306
        if c.convolutional or c.second_order or c.opcode not in (0, 1):
            raise ValueError("Unimplemented connection type!")
        st, m = self.neuron[c.to], self.matrix[c]
        L.sg_upd_spnet(c.rows, _p(c.dst), _p(c.ptr), _p(c.from_idx), _p(c.w_idx),
                       c.frm.output_type, int(c.opcode == 1), ctypes.c_float(c.learning_rate),
                       ctypes.c_float(c.max_weight), _p(st["post trace"]), _p(st["time since spike"]),
                       _p(st["output"][:c.to.size]), _p(m["time since spike"]), _p(m["weights"]),
                       _p(m["presyn trace"]), _p(m["weight derivative"]))

    def _activate_nvm(self, L, c, st, m, src, geo, reg):
        """NVM activator choice (nvm_attributes.cpp:163-187,
        nvm_compare_attributes.cpp:60-69) and the layer's gates."""
        if c.second_order:
            raise ValueError("Unimplemented connection type!")
        l = c.to
        flag = lambda k: c.p.get(k, "false") == "true"
        kinds = [("decay", 0), ("gate", 1), ("learning", 2), ("noise", 3)]
        if not (l.model == "nvm_compare" and c.plastic):
            for name, g in kinds:
                if flag(name):
                    if c.c.type == 1:   # a subset window (an empty one writes nothing)
                        gv = np.float32(lib_gate(L, c, src))
                        if g == 0:
                            l.gates[0] = np.float32(1.0) - gv
                        else:
                            l.gates[{1: 0, 2: 1, 3: 2}[g]] = gv
                    return
            if flag("context"):
                L.sg_act_nvm_context(c.frm.size, _p(src), c.frm.output_type, c.delay, c.opcode,
                                     _p(m["weights"]), ctypes.c_float(l.gates[0]), _p(st["context"]))
                return
        if l.model == "nvm_compare" and c.plastic:
            kind = 3
        elif c.plastic:
            kind = 2
        elif flag("gated"):
            kind = 1
        else:
            kind = 0
        truth = st["true_state"] if l.model == "nvm_compare" else st["state"]
        L.sg_act_nvm(kind, *geo, _p(src), c.frm.output_type, c.delay, c.opcode, _p(m["weights"]),
                     _p(reg), ctypes.c_float(l.gates[0]), ctypes.c_float(l.gates[1]),
                     _p(st["state"]), _p(st["context"]), _p(truth),
                     ctypes.c_float(c.p.get_float("norm", 1.0)), c.num_weights // l.size,
                     ctypes.c_float(getattr(l, "tolerance", 0.0)))


def lib_gate(L, c, src):
    L.sg_nvm_gate.restype = ctypes.c_float
    return L.sg_nvm_gate(ctypes.byref(c.c), _p(src), c.frm.output_type, c.delay,
                         int(c.p.get("decay", "false") == "true"))
