"""Saves and loads network states with the reference's own CPU library (test
infrastructure for the state-interchange tests, run in a child process so
that the two libraries never share a process).

  python tests/golden/ref_state.py save <case> <steps> <state file> <npz>
  python tests/golden/ref_state.py load <case> <state file> <npz>

`save` runs the case for `steps` steps (injections and inputs as in the
fixtures, one OpenMP thread) and saves the state; `load` builds the case's
network fresh and loads the state.  Both then write every array the case
compares, as read through the reference's getters, to the npz.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)


def state_keys(case):
    """(kind, ..., key) of the arrays compared: every layer's input and output
    and each connection's weights, plus the case's final arrays."""
    keys = []
    for st in case.net["structures"]:
        for l in st["layers"]:
            keys += [("neuron", st["name"], l["name"], "input"),
                     ("neuron", st["name"], l["name"], "output")]
    for c in case.net["connections"]:
        keys.append(("matrix", c["name"], "weights"))
    for k in case.final:
        if tuple(k) not in keys:
            keys.append(tuple(k))
    return keys


def dump(net, case, path):
    out = {}
    for key in state_keys(case):
        if key[0] == "neuron":
            a = net.get_neuron_data(key[1], key[2], key[3])
        else:
            a = net.get_weight_matrix(key[1], key[2])
        a = np.array(a.to_np_array(), copy=True)
        out["/".join(key)] = a.view(np.uint32) if a.dtype == np.float32 else a
    np.savez(path, **out)


def main(argv):
    from cases import CASES
    from make_golden import load_reference_syngen
    from tests.harness import case_sizes
    from tests.golden.cases import callback_injections
    sg = load_reference_syngen()
    case = CASES[argv[1]]
    sizes = case_sizes(case)
    net_dict, injections, weight_arrays, delay_arrays = callback_injections(
        case.net, case.injections(sizes))

    def weight_cb(ID, size, weights):
        sg.FloatArray(size, weights).to_np_array()[:] = weight_arrays[ID]

    def delay_cb(ID, size, weights, delays):
        sg.IntArray(size, delays).to_np_array()[:] = delay_arrays[ID]

    sg._delay_weight_callbacks = {}
    sg.create_weight_callback("golden_weight", weight_cb)
    sg.create_delay_weight_callback("golden_delay", delay_cb)
    net = sg.Network(net_dict)
    if argv[0] == "load":
        net.build_state()
        net.load_state(argv[2])
        dump(net, case, argv[3])
        return
    steps = int(argv[2])
    net.build_state()
    for key, arr in injections.items():
        if key[0] == "neuron":
            dst = net.get_neuron_data(key[1], key[2], key[3]).to_np_array()
        else:
            dst = net.get_weight_matrix(key[1], key[2]).to_np_array()
        dst.view(arr.dtype)[:] = arr
    inputs = case.input_arrays(sizes, steps)
    in_layers = sorted(case.inputs)
    step = {"in": 0}

    def in_cb(ID, size, ptr):
        sg.FloatArray(size, ptr).to_np_array()[:] = inputs[step["in"]][in_layers[ID]]
        if ID == len(in_layers) - 1:
            step["in"] += 1

    sg.create_io_callback("golden_in", in_cb)
    structs = {l["name"]: st["name"] for st in case.net["structures"] for l in st["layers"]}
    modules = []
    if in_layers:
        modules.append({"type": "callback", "layers": [
            {"structure": structs[l], "layer": l, "input": True, "function": "golden_in", "id": i}
            for i, l in enumerate(in_layers)]})
    if steps > 0:
        net.run(sg.Environment({"modules": modules}),
                {"iterations": steps, "multithreaded": False, "worker threads": 0,
                 "learning flag": case.learning})
    net.save_state(argv[3])
    dump(net, case, argv[4])


if __name__ == "__main__":
    main(sys.argv[1:])
