"""Python front-end of the GB300 simulation-cycle library.

Same public surface as the reference front-end (lib/syngen.py): array
wrappers, ``Properties``, ``Network``, ``Environment``, named callbacks,
factories and the module builders, bound over ctypes to the C-ABI declared in
include/syngen.h.  By default it loads the in-tree GB300 library; set
``SYNGEN_LIB`` to a path to bind another build of the same C-ABI (for example
the reference's own CPU library).  Importing fails loudly when the library has
not been built -- there is no fallback.
"""
import ctypes
import os
from collections import OrderedDict
from copy import deepcopy
from ctypes import (CFUNCTYPE, POINTER, Structure, c_bool, c_char, c_char_p, c_float, c_int,
                    c_longlong, c_uint, c_ulonglong, c_void_p, cast, string_at)
from json import dumps
from math import exp

from numpy import copyto
from numpy.ctypeslib import as_array

_HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_LIB = os.path.join(_HERE, "_build", "libsyngen.so")


class CArray(Structure):
    """ARRAY struct of the C-ABI (extern.h:14-19)."""
    _fields_ = [("size", c_int), ("type", c_uint), ("data", c_void_p), ("owner", c_bool)]


class PArray:
    """Typed view of a C array."""

    def __init__(self, size, ptr):
        self.size = size
        self.data = ptr

    def __getitem__(self, i):
        return self.data[i]

    def __setitem__(self, i, v):
        self.data[i] = v

    def __iter__(self):
        for i in range(self.size):
            yield self.data[i]

    def __len__(self):
        return self.size

    def is_void(self):
        return False

    def to_np_array(self):
        return as_array(self.data, shape=(self.size,))

    def copy_from(self, arr):
        copyto(self.to_np_array(), arr)


class FloatArray(PArray):
    def __init__(self, size, ptr):
        super().__init__(size, cast(ptr, POINTER(c_float)))

    def to_list(self):
        return [float(x) for x in self]


class IntArray(PArray):
    def __init__(self, size, ptr):
        super().__init__(size, cast(ptr, POINTER(c_int)))

    def to_list(self):
        return [int(x) for x in self]


class StringArray(PArray):
    def __init__(self, size, ptr):
        super().__init__(size, cast(ptr, POINTER(POINTER(c_char))))


class VoidArray(PArray):
    def __init__(self, size, ptr):
        super().__init__(size, cast(ptr, POINTER(c_void_p)))

    def is_void(self):
        return True


_ARRAY_TYPES = {1: FloatArray, 2: IntArray, 3: StringArray, 4: VoidArray, 5: VoidArray}


def build_array(base):
    """Wraps a CArray by its POINTER_TYPE (extern.h:6-12)."""
    return _ARRAY_TYPES[base.type](base.size, base.data)


def _load_library(path=None):
    path = path or os.environ.get("SYNGEN_LIB") or DEFAULT_LIB
    if not os.path.exists(path):
        raise ImportError("GB300 syngen library not built (%s); run "
                          "`python -c 'import __graft_entry__ as g; g.build()'`" % path)
    lib = ctypes.CDLL(path)
    sig = {
        "free_array": ((CArray,), None), "free_array_deep": ((CArray,), None),
        "create_properties": ((), c_void_p),
        "add_property": ((c_void_p, c_char_p, c_char_p), None),
        "add_child": ((c_void_p, c_char_p, c_void_p), None),
        "add_to_array": ((c_void_p, c_char_p, c_char_p), None),
        "add_to_child_array": ((c_void_p, c_char_p, c_void_p), None),
        "get_keys": ((c_void_p,), CArray), "get_child_keys": ((c_void_p,), CArray),
        "get_array_keys": ((c_void_p,), CArray), "get_child_array_keys": ((c_void_p,), CArray),
        "get_property": ((c_void_p, c_char_p), c_char_p),
        "get_child": ((c_void_p, c_char_p), c_void_p),
        "get_array": ((c_void_p, c_char_p), CArray),
        "get_child_array": ((c_void_p, c_char_p), CArray),
        "create_environment": ((c_void_p,), c_void_p), "load_env": ((c_char_p,), c_void_p),
        "save_env": ((c_void_p, c_char_p), c_bool),
        "create_network": ((c_void_p,), c_void_p), "load_net": ((c_char_p,), c_void_p),
        "save_net": ((c_void_p, c_char_p), c_bool),
        "build_state": ((c_void_p,), c_void_p), "build_load_state": ((c_void_p, c_char_p), c_void_p),
        "load_state": ((c_void_p, c_char_p), c_bool), "save_state": ((c_void_p, c_char_p), c_bool),
        "get_neuron_data": ((c_void_p, c_char_p, c_char_p, c_char_p), CArray),
        "get_layer_data": ((c_void_p, c_char_p, c_char_p, c_char_p), CArray),
        "get_connection_data": ((c_void_p, c_char_p, c_char_p), CArray),
        "get_weight_matrix": ((c_void_p, c_char_p, c_char_p), CArray),
        "run": ((c_void_p, c_void_p, c_void_p, c_void_p), c_void_p),
        "destroy": ((c_void_p,), None), "destroy_network": ((c_void_p,), None),
        "destroy_environment": ((c_void_p,), None), "destroy_state": ((c_void_p,), None),
        "destroy_properties": ((c_void_p,), None),
        "get_cpu": ((), c_int), "get_gpus": ((), CArray), "get_all_devices": ((), CArray),
        "set_suppress_output": ((c_bool,), None), "set_warnings": ((c_bool,), None),
        "set_debug": ((c_bool,), None), "interrupt_engine": ((), None),
        "add_io_callback": ((c_char_p, c_longlong), None),
        "add_weight_callback": ((c_char_p, c_longlong), None),
        "add_indices_weight_callback": ((c_char_p, c_longlong), None),
        "add_distance_weight_callback": ((c_char_p, c_longlong), None),
        "add_delay_weight_callback": ((c_char_p, c_longlong), None),
        "get_mpi_rank": ((), c_int), "get_mpi_size": ((), c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if hasattr(lib, "sg_last_error"):
        lib.sg_last_error.restype = c_char_p
        lib.sg_set_seed.argtypes = (c_ulonglong,)
        lib.sg_engine_create.argtypes = (c_void_p, c_void_p, c_void_p, c_void_p)
        lib.sg_engine_create.restype = c_void_p
        lib.sg_engine_step.argtypes = (c_void_p, c_longlong)
        lib.sg_engine_step.restype = c_longlong
        lib.sg_engine_stream.argtypes = (c_void_p,)
        lib.sg_engine_stream.restype = c_void_p
        lib.sg_engine_report.argtypes = (c_void_p,)
        lib.sg_engine_report.restype = c_void_p
        lib.sg_engine_destroy.argtypes = (c_void_p,)
    if hasattr(lib, "sg_batch_create"):
        lib.sg_batch_create.argtypes = (POINTER(BatchInstance), c_int, c_int, c_int)
        lib.sg_batch_create.restype = c_void_p
        lib.sg_batch_step.argtypes = (c_void_p, c_longlong)
        lib.sg_batch_step.restype = c_int
        lib.sg_batch_read.argtypes = (c_void_p, c_int, c_char_p, c_void_p, c_longlong)
        lib.sg_batch_read.restype = c_int
        lib.sg_batch_report.argtypes = (c_void_p,)
        lib.sg_batch_report.restype = c_void_p
        lib.sg_batch_stream.argtypes = (c_void_p,)
        lib.sg_batch_stream.restype = c_void_p
        lib.sg_batch_synchronize.argtypes = (c_void_p,)
        lib.sg_batch_synchronize.restype = c_int
        lib.sg_batch_destroy.argtypes = (c_void_p,)
    if hasattr(lib, "sg_rate_forward"):
        lib.sg_rate_workspace_bytes.argtypes = (POINTER(RateShape),)
        lib.sg_rate_workspace_bytes.restype = c_longlong
        lib.sg_rate_forward.argtypes = (POINTER(RateShape),) + (c_void_p,) * 9
        lib.sg_rate_forward.restype = c_int
        lib.sg_rate_backward.argtypes = ((POINTER(RateShape),) + (c_void_p,) * 5 + (c_float,)
                                         + (c_void_p,) * 6)
        lib.sg_rate_backward.restype = c_int
    return lib, path


class RateShape(Structure):
    """SgRateShape of include/syngen.h."""
    _fields_ = [("layers", c_int), ("rows", c_int), ("cols", c_int), ("field", c_int),
                ("outputs", c_int), ("batch", c_int), ("steps", c_int), ("checkpoint", c_int),
                ("dt", c_float)]


class BatchInstance(Structure):
    """SgBatchInstance of include/syngen.h: one instance of a batch."""
    _fields_ = [("rows", c_int), ("cols", c_int), ("a", c_float), ("b", c_float),
                ("c", c_float), ("d", c_float), ("v0", c_float), ("seed", c_ulonglong),
                ("input_rate", c_float), ("input_value", c_float), ("conv_field", c_int),
                ("conv_wmax", c_float), ("conv_stp_w", c_float), ("conv_conductance", c_float),
                ("fc_wmax", c_float), ("fc_density", c_float), ("fc_stp_w", c_float),
                ("fc_conductance", c_float), ("fc_max_delay", c_int)]


_syn, LIB_PATH = _load_library()


def last_error():
    """Message of the last failed C-ABI call (GB300 library only)."""
    if hasattr(_syn, "sg_last_error"):
        return _syn.sg_last_error().decode("utf-8")
    return ""


def set_seed(seed):
    """Seeds the random weight / parameter / noise initialisers."""
    _syn.sg_set_seed(int(seed))


# --- simple functions -------------------------------------------------------
def _int_list(arr_obj):
    out = build_array(arr_obj).to_list() if arr_obj.data else []
    _syn.free_array(arr_obj)
    return out


def get_cpu():
    return _syn.get_cpu()


def get_gpus():
    return _int_list(_syn.get_gpus())


def get_all_devices():
    return _int_list(_syn.get_all_devices())


def set_suppress_output(val):
    _syn.set_suppress_output(val)


def set_warnings(val):
    _syn.set_warnings(val)


def set_debug(val):
    _syn.set_debug(val)


def interrupt_engine():
    _syn.interrupt_engine()


# --- named callbacks ----------------------------------------------------------
_io_callbacks = {}
_weight_callbacks = {}
_indices_weight_callbacks = {}
_distance_weight_callbacks = {}
_delay_weight_callbacks = {}
_callback_config_map = {}

_IO_T = CFUNCTYPE(None, c_int, c_int, c_void_p)
_INDICES_T = CFUNCTYPE(None, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p)
_PAIR_T = CFUNCTYPE(None, c_int, c_int, c_void_p, c_void_p)


def make_callback_id(config):
    key = len(_callback_config_map)
    _callback_config_map[key] = config
    return key


def get_config(ID):
    return _callback_config_map[ID]


def _register(table, ctype, adder, name, f):
    cb = ctype(f)
    addr = cast(cb, c_void_p).value
    table[name] = (cb, addr)      # keep the thunk alive
    adder(name.encode("utf-8"), addr)


def create_io_callback(name, f):
    _register(_io_callbacks, _IO_T, _syn.add_io_callback, name, f)


def create_weight_callback(name, f):
    _register(_weight_callbacks, _IO_T, _syn.add_weight_callback, name, f)


def create_indices_weight_callback(name, f):
    _register(_indices_weight_callbacks, _INDICES_T, _syn.add_indices_weight_callback, name, f)


def create_distance_weight_callback(name, f):
    _register(_distance_weight_callbacks, _PAIR_T, _syn.add_distance_weight_callback, name, f)


def create_delay_weight_callback(name, f):
    _register(_delay_weight_callbacks, _PAIR_T, _syn.add_delay_weight_callback, name, f)


# --- properties -----------------------------------------------------------------
def _to_str(v):
    if isinstance(v, bool):
        return "true" if v else "false"
    return str(v)


def _strings(arr_obj):
    arr = build_array(arr_obj)
    out = [string_at(cast(arr.data[i], c_char_p)).decode("utf-8") for i in range(arr.size)]
    return out


_EMPTY = object()


class Properties:
    """String-keyed property tree; built from a dict, or read from a C handle."""

    def __init__(self, props=_EMPTY):
        self.properties = OrderedDict()
        self.children = OrderedDict()
        self.arrays = OrderedDict()
        self.child_arrays = OrderedDict()
        self.obj = None          # stays None for a failed call's NULL handle
        if props is _EMPTY:
            props = {}
        if isinstance(props, dict):
            self.obj = _syn.create_properties()
            for k, v in props.items():
                if v is None:
                    continue
                if isinstance(v, dict):
                    self.add_child(k, v)
                elif isinstance(v, list):
                    for x in v:
                        if isinstance(x, dict):
                            self.add_to_child_array(k, x)
                        else:
                            self.add_to_array(k, _to_str(x))
                else:
                    self.add_property(k, v)
        elif isinstance(props, int):
            self.obj = props
            self._read(props)

    def _read(self, handle):
        keys_obj = _syn.get_keys(handle)
        for key in _strings(keys_obj):
            self.properties[key] = _syn.get_property(handle, key.encode("utf-8")).decode("utf-8")
        _syn.free_array_deep(keys_obj)
        keys_obj = _syn.get_child_keys(handle)
        for key in _strings(keys_obj):
            self.children[key] = Properties(_syn.get_child(handle, key.encode("utf-8")))
        _syn.free_array_deep(keys_obj)
        keys_obj = _syn.get_array_keys(handle)
        for key in _strings(keys_obj):
            arr_obj = _syn.get_array(handle, key.encode("utf-8"))
            self.arrays.setdefault(key, []).extend(_strings(arr_obj))
            _syn.free_array_deep(arr_obj)
        _syn.free_array_deep(keys_obj)
        keys_obj = _syn.get_child_array_keys(handle)
        for key in _strings(keys_obj):
            arr_obj = _syn.get_child_array(handle, key.encode("utf-8"))
            arr = build_array(arr_obj)
            self.child_arrays.setdefault(key, []).extend(
                Properties(arr.data[i]) for i in range(arr.size))
            _syn.free_array(arr_obj)
        _syn.free_array_deep(keys_obj)

    def to_dict(self):
        out = OrderedDict(self.properties)
        for k, v in self.children.items():
            out[k] = v.to_dict()
        for k, v in self.arrays.items():
            out[k] = [str(p) for p in v]
        for k, v in self.child_arrays.items():
            out[k] = [p.to_dict() for p in v]
        return out

    def __str__(self):
        return dumps(self.to_dict(), indent=4)

    def add_property(self, key, val):
        self.properties[key] = val
        _syn.add_property(self.obj, key.encode("utf-8"), _to_str(val).encode("utf-8"))

    def add_child(self, key, child):
        child = Properties(child)
        self.children[key] = child
        _syn.add_child(self.obj, key.encode("utf-8"), child.obj)

    def add_to_array(self, key, val):
        self.arrays.setdefault(key, []).append(val)
        _syn.add_to_array(self.obj, key.encode("utf-8"), val.encode("utf-8"))

    def add_to_child_array(self, key, dictionary):
        props = Properties(dictionary)
        self.child_arrays.setdefault(key, []).append(props)
        _syn.add_to_child_array(self.obj, key.encode("utf-8"), props.obj)

    def free(self):
        if _syn is not None and self.obj is not None:
            _syn.destroy(self.obj)
            self.obj = None


class Environment:
    def __init__(self, env):
        self.props = None
        if isinstance(env, str):
            self.obj = _syn.load_env(env.encode("utf-8"))
        elif isinstance(env, dict):
            self.props = Properties(env)
            self.obj = _syn.create_environment(self.props.obj)
        else:
            self.obj = None

    def save(self, filename):
        return _syn.save_env(self.obj, filename.encode("utf-8"))

    def free(self):
        if self.props is not None:
            self.props.free()
            self.props = None
        _syn.destroy_environment(self.obj)
        self.obj = None


class Network:
    def __init__(self, net):
        self.props = None
        self.state = None
        if isinstance(net, str):
            self.obj = _syn.load_net(net.encode("utf-8"))
        elif isinstance(net, dict):
            self.props = Properties(net)
            self.obj = _syn.create_network(self.props.obj)
        else:
            self.obj = None

    def save(self, filename):
        return _syn.save_net(self.obj, filename.encode("utf-8"))

    def free(self):
        if self.props is not None:
            self.props.free()
            self.props = None
        if self.state is not None:
            _syn.destroy_state(self.state)
            self.state = None
        _syn.destroy_network(self.obj)
        self.obj = None

    def build_state(self, filename=None):
        if self.state is not None:
            _syn.destroy_state(self.state)
        if filename is None:
            self.state = _syn.build_state(self.obj)
        else:
            self.state = _syn.build_load_state(self.obj, filename.encode("utf-8"))

    def load_state(self, filename):
        if self.state is None:
            self.build_state(filename)
        else:
            _syn.load_state(self.state, filename.encode("utf-8"))

    def save_state(self, filename):
        if self.state is None:
            self.build_state()
        _syn.save_state(self.state, filename.encode("utf-8"))

    def get_neuron_data(self, structure, layer, key):
        if self.state is None:
            self.build_state()
        return build_array(_syn.get_neuron_data(self.state, structure.encode("utf-8"),
                                                layer.encode("utf-8"), key.encode("utf-8")))

    def get_layer_data(self, structure, layer, key):
        if self.state is None:
            self.build_state()
        return build_array(_syn.get_layer_data(self.state, structure.encode("utf-8"),
                                               layer.encode("utf-8"), key.encode("utf-8")))

    def get_connection_data(self, structure, connection, key):
        if self.state is None:
            self.build_state()
        return build_array(_syn.get_connection_data(self.state, connection.encode("utf-8"),
                                                    key.encode("utf-8")))

    def get_weight_matrix(self, connection, key="weights"):
        if self.state is None:
            self.build_state()
        return build_array(_syn.get_weight_matrix(self.state, connection.encode("utf-8"),
                                                  key.encode("utf-8")))

    def run(self, environment, args=None):
        if self.state is None:
            self.build_state()
        if not isinstance(environment, Environment):
            environment = Environment(environment)
        if not isinstance(args, Properties):
            args = Properties(args or {})
        report = _syn.run(self.obj, environment.obj, self.state, args.obj)
        if report is None:
            print("Failed to run network!", last_error())
        return Properties(report)


class Engine:
    """A run that stays open: step it repeatedly on the same state (GB300
    library extension, sg_engine_* in include/syngen.h)."""

    def __init__(self, network, environment=None, args=None):
        if network.state is None:
            network.build_state()
        self.network = network
        self.environment = environment if isinstance(environment, Environment) else \
            Environment(environment or {"modules": []})
        self.args = args if isinstance(args, Properties) else Properties(args or {})
        self.obj = _syn.sg_engine_create(network.obj, self.environment.obj, network.state,
                                         self.args.obj)
        if not self.obj:
            raise RuntimeError("engine creation failed: " + last_error())

    def step(self, n):
        done = _syn.sg_engine_step(self.obj, int(n))
        if done < 0:
            raise RuntimeError("engine step failed: " + last_error())
        return done

    @property
    def stream(self):
        """cudaStream_t (as an int) that every kernel of this engine runs on."""
        return _syn.sg_engine_stream(self.obj)

    def report(self):
        return Properties(_syn.sg_engine_report(self.obj))

    def close(self):
        if self.obj:
            _syn.sg_engine_destroy(self.obj)
            self.obj = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Batch:
    """Many independent Izhikevich instances advanced together (sg_batch_* in
    include/syngen.h).  ``instances`` is a sequence of dicts with the fields of
    ``BatchInstance``; ``tile`` = (rows, colblocks) fixes the step kernel's work
    unit, None lets the autotuner choose."""

    def __init__(self, instances, tile=None):
        n = len(instances)
        arr = (BatchInstance * n)()
        for i, spec in enumerate(instances):
            for k, v in spec.items():
                setattr(arr[i], k, v)
        self.sizes = [(s["rows"], s["cols"]) for s in instances]
        tr, tc = tile if tile else (0, 0)
        self.obj = _syn.sg_batch_create(arr, n, int(tr), int(tc))
        if not self.obj:
            raise RuntimeError("batch creation failed: " + last_error())

    def step(self, n):
        if _syn.sg_batch_step(self.obj, int(n)) != 0:
            raise RuntimeError("batch step failed: " + last_error())

    def read(self, instance, key):
        """Host copy of "voltage", "recovery" (float32) or "output" (uint32)."""
        import numpy as np
        rows, cols = self.sizes[instance]
        out = np.empty(rows * cols, np.uint32 if key == "output" else np.float32)
        if _syn.sg_batch_read(self.obj, int(instance), key.encode("utf-8"),
                              out.ctypes.data, out.size) != 0:
            raise RuntimeError("batch read failed: " + last_error())
        return out

    @property
    def stream(self):
        return _syn.sg_batch_stream(self.obj)

    def synchronize(self):
        if _syn.sg_batch_synchronize(self.obj) != 0:
            raise RuntimeError("batch synchronize failed")

    def report(self):
        return Properties(_syn.sg_batch_report(self.obj))

    def close(self):
        if self.obj:
            _syn.sg_batch_destroy(self.obj)
            self.obj = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class RateNetwork:
    """Differentiable leaky-integrator rate network (sg_rate_* in
    include/syngen.h): ``layers`` layers of rows x cols neurons, convergent
    field x field connections between consecutive layers, a readout of the
    last layer, per-layer learnable time constants.  ``loss`` is a
    torch.autograd-aware call whose backward pass is the library's hand-written
    adjoint with a checkpoint every ``checkpoint`` steps."""

    def __init__(self, layers=3, rows=64, cols=64, field=5, outputs=10, batch=64, steps=100,
                 dt=1.0, checkpoint=10):
        self.shape = RateShape(layers, rows, cols, field, outputs, batch, steps, checkpoint, dt)
        n = _syn.sg_rate_workspace_bytes(ctypes.byref(self.shape))
        if n < 0:
            raise ValueError("invalid rate network: " + last_error())
        self.workspace_bytes = int(n)
        self.neurons = rows * cols

    def parameter_shapes(self):
        s = self.shape
        return {"x": (s.steps, s.batch, self.neurons),
                "weights": (max(s.layers - 1, 0), self.neurons, s.field * s.field),
                "readout": (s.outputs, self.neurons), "tau": (s.layers,),
                "target": (s.batch, s.outputs)}

    def loss(self, x, weights, readout, tau, target):
        return _rate_loss_function().apply(self, x, weights, readout, tau, target)

    def _check(self, **tensors):
        import torch
        for name, shp in self.parameter_shapes().items():
            t = tensors[name]
            if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32
                    and t.is_contiguous() and tuple(t.shape) == shp):
                raise ValueError("%s must be a contiguous float32 CUDA tensor of shape %s"
                                 % (name, shp))

    def _forward(self, x, weights, readout, tau, target, y=None):
        import torch
        self._check(x=x, weights=weights, readout=readout, tau=tau, target=target)
        ws = torch.empty(self.workspace_bytes // 4, dtype=torch.float32, device=x.device)
        loss = torch.empty((), dtype=torch.float32, device=x.device)
        rc = _syn.sg_rate_forward(ctypes.byref(self.shape), x.data_ptr(),
                                  weights.data_ptr() if weights.numel() else None,
                                  readout.data_ptr(), tau.data_ptr(), target.data_ptr(),
                                  y.data_ptr() if y is not None else None, loss.data_ptr(),
                                  ws.data_ptr(), torch.cuda.current_stream(x.device).cuda_stream)
        if rc != 0:
            raise RuntimeError("rate forward failed: " + last_error())
        return loss, ws

    def _backward(self, ws, grad_loss, x, weights, readout, tau, target, want_dx=True):
        import torch
        dw = torch.empty_like(weights)
        dR = torch.empty_like(readout)
        dtau = torch.empty_like(tau)
        dx = torch.empty_like(x) if want_dx else None
        rc = _syn.sg_rate_backward(ctypes.byref(self.shape), x.data_ptr(),
                                   weights.data_ptr() if weights.numel() else None,
                                   readout.data_ptr(), tau.data_ptr(), target.data_ptr(),
                                   float(grad_loss), ws.data_ptr(),
                                   dw.data_ptr() if weights.numel() else None, dR.data_ptr(),
                                   dtau.data_ptr(), dx.data_ptr() if dx is not None else None,
                                   torch.cuda.current_stream(x.device).cuda_stream)
        if rc != 0:
            raise RuntimeError("rate backward failed: " + last_error())
        return dx, dw, dR, dtau


_RATE_FN = []


def _rate_loss_function():
    """torch.autograd.Function over sg_rate_forward / sg_rate_backward (built
    on first use so that importing this module does not import torch)."""
    if _RATE_FN:
        return _RATE_FN[0]
    import torch

    class RateLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, net, x, weights, readout, tau, target):
            loss, ws = net._forward(x, weights, readout, tau, target)
            ctx.net, ctx.ws = net, ws
            ctx.save_for_backward(x, weights, readout, tau, target)
            return loss

        @staticmethod
        def backward(ctx, grad_loss):
            x, weights, readout, tau, target = ctx.saved_tensors
            dx, dw, dR, dtau = ctx.net._backward(ctx.ws, float(grad_loss), x, weights, readout,
                                                 tau, target, want_dx=ctx.needs_input_grad[1])
            return None, dx, dw, dR, dtau, None

    _RATE_FN.append(RateLoss)
    return RateLoss


def fill_in(defaults, props):
    new_props = deepcopy(props)
    for k, v in defaults.items():
        if isinstance(v, dict):
            new_props[k] = fill_in(v, new_props[k]) if k in new_props else deepcopy(v)
        elif k not in new_props:
            new_props[k] = deepcopy(v)
    return new_props


class PropertiesFactory:
    def __init__(self, defaults=None, func=None):
        if defaults is None and func is None:
            raise ValueError
        self.set_defaults(defaults)
        self.set_func(func)

    def set_defaults(self, defaults):
        if defaults is not None and not isinstance(defaults, dict):
            raise ValueError
        self.defaults = defaults

    def set_func(self, func):
        if func is not None and not callable(func):
            raise ValueError
        self.func = func

    def build(self, props=None):
        new_props = deepcopy(props or {})
        if self.defaults is not None:
            new_props = fill_in(self.defaults, new_props)
        if self.func is not None:
            self.func(new_props)
        return new_props


class LayerFactory(PropertiesFactory):
    pass


class ConnectionFactory(PropertiesFactory):
    def build(self, from_layer, to_layer, props=None):
        new_props = deepcopy(props or {})
        if self.defaults is not None:
            new_props = fill_in(self.defaults, new_props)
        if self.func is not None:
            self.func(from_layer, to_layer, new_props)
        return new_props


def make_custom_input_module(structure, layer_names, name, cb, clear=True):
    def custom_callback(ID, size, ptr):
        cb(layer_names[ID], FloatArray(size, ptr).to_np_array())
    create_io_callback(name, custom_callback)
    return {"type": "callback", "clear": clear,
            "layers": [{"structure": structure, "layer": l, "input": True, "function": name,
                        "id": i} for i, l in enumerate(layer_names)]}


def make_custom_output_module(structure, layer_names, name, cb):
    def custom_callback(ID, size, ptr):
        cb(layer_names[ID], FloatArray(size, ptr).to_np_array())
    create_io_callback(name, custom_callback)
    return {"type": "callback",
            "layers": [{"structure": structure, "layer": l, "output": True, "function": name,
                        "id": i} for i, l in enumerate(layer_names)]}


# --- common weight callbacks ---------------------------------------------------------
def gauss(dist, peak, sig, norm=False):
    inv_sqrt_2pi = 0.3989422804014327
    a = dist / sig
    return peak * (1.0 if norm else inv_sqrt_2pi / sig) * exp(-0.5 * a * a)


def diff_gauss(dist, peak, sig, norm=False):
    v = gauss(dist, peak, sig, False) - gauss(dist, peak, sig * 1.6, False)
    if norm:
        inv_sqrt_2pi = 0.3989422804014327
        v = v / ((inv_sqrt_2pi / sig) - (inv_sqrt_2pi / (sig * 1.6)))
    return v


def _dist_callback(shape):
    def cb(ID, size, weights, distances):
        w = FloatArray(size, weights)
        d = FloatArray(size, distances)
        sigma = max(d.data[i] for i in range(size)) / 2
        if sigma != 0:
            for i in range(size):
                w.data[i] = shape(d.data[i], w.data[i], sigma, True)
    return cb


gaussian_dist_callback = _dist_callback(gauss)
mexican_hat_dist_callback = _dist_callback(diff_gauss)
create_distance_weight_callback("gaussian", gaussian_dist_callback)
create_distance_weight_callback("mexican_hat", mexican_hat_dist_callback)


def get_dsst_params(num_rows=8, cell_res=8):
    num_cols = 18
    cell_rows = 2 * cell_res + 1
    spacing = cell_res / 4
    input_rows = (num_rows + 2) * (cell_rows + spacing) - spacing
    input_cols = num_cols * (cell_res + spacing) - spacing
    return {"columns": num_cols, "rows": num_rows, "cell columns": cell_res,
            "cell rows": cell_rows, "spacing": spacing, "input rows": input_rows,
            "input columns": input_cols, "focus rows": input_rows - cell_rows,
            "focus columns": input_cols - cell_res}


def get_mpi_rank():
    return _syn.get_mpi_rank()


def get_mpi_size():
    return _syn.get_mpi_size()
