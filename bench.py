"""Benchmark of the GB300 simulation cycle (one JSON line on rank 0).

Default workload (``iz_plastic``): three 256x256 Izhikevich layers (80%
regular / 20% fast spiking), L1->L2 convergent 9x9 with STDP, L2->L3
divergent 3x3 stride 2, L3->L1 one-to-one, a 4096x4096 subset projection,
delays U{0..3}, a 5 Hz Poisson drive generated on the device; one bench step
is 1000 timesteps.  Metric: synapse updates per second (one (destination,
weight) visit in an activator or updater in one timestep).  The network and
its injected weights, delays and per-neuron parameters are those of the
parity case at the same size (tests/golden/configs.py).

On one GPU the line also nests the other measured configurations under
"configs" (each from its own child run of this script): ``iz_c0`` (32x32
Izhikevich), ``gol`` (game of life 2048x2048, 10,000 timesteps per step),
``batched`` (256 instances) and ``rate_adjoint`` (differentiable rate
network), each with its roofline, CPU baseline and end-to-end figure.

  python bench.py [--gpus N] [--steps K] [--warmup W]
                  [--workload iz_plastic|iz_c0|gol|batched|rate_adjoint|spnet_sparse]
  python bench.py --impl reference ...   # the reference's own CPU path

Timing: each step is bracketed by CUDA events recorded on the stream the
library launches every kernel on; L2 is flushed (a 256 MiB buffer is written)
between steps, outside the events.  Under torchrun each rank runs an
independent replica on its own GPU (the single-network cycle does not shard);
value is the sum over ranks of units over the max over ranks of time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libsyngen.so")
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC = os.path.join(ROOT, "profiles", "traffic.json")
FALLBACK_HBM_GBS = 6800.0


# ---------------------------------------------------------------------------
# Workloads (synthetic, seeded)
# ---------------------------------------------------------------------------
# Timesteps per launch of the whole-run game_of_life kernel (the library's
# default, or its SG_GOL_STEPS_PER_LAUNCH override).
GOL_STEPS_PER_LAUNCH = int(os.environ.get("SG_GOL_STEPS_PER_LAUNCH", "12"))


def gol_workload(side=2048):
    import numpy as np
    net = {"structures": [{"name": "g", "type": "parallel", "layers": [
        {"name": "board", "neural model": "game_of_life", "rows": side, "columns": side,
         "survival_min": 2, "survival_max": 3, "birth_min": 3, "birth_max": 3}]}],
        "connections": [{"name": "nbr", "from layer": "board", "to layer": "board",
                         "type": "convergent", "convolutional": True, "plastic": False,
                         "opcode": "add",
                         "weight config": {"type": "flat", "weight": 1.0, "diagonal": False},
                         "arborized config": {"field size": 3, "wrap": True}}]}
    n = side * side

    def inject(net_obj):
        rng = np.random.default_rng(1)
        out = net_obj.get_neuron_data("g", "board", "output").to_np_array().view(np.uint32)
        out[:] = (rng.random(n) < 0.3).astype(np.uint32) << np.uint32(31)

    def result(net_obj):
        return net_obj.get_neuron_data("g", "board", "output").to_np_array()

    return {
        "name": "gol",
        "desc": "game_of_life %dx%d toroidal, 3x3 convergent wrap, B3/S23, p_alive=0.3 seed 1" % (side, side),
        "net": net, "inject": inject, "result": result,
        "timesteps": 10000,                  # per bench step: the full configured run
        "units_per_timestep": 9 * n,
        "unit": "synapse-updates/s",
        "dtype": "u32",
        # Whole runs on bit planes: one launch advances GOL_STEPS_PER_LAUNCH
        # timesteps; per timestep and cell a step reads the newest and the
        # oldest history bit and writes one new bit (3 bits); the word layout
        # would move 8 B.
        "kernel": "k_gol_strips_steps (%d timesteps per launch)" % GOL_STEPS_PER_LAUNCH,
        "profile_group": "game_of_life.advance",
        "steps_per_launch": GOL_STEPS_PER_LAUNCH,
        "timestep_bytes": 3 * n // 8,
        "word_layout_timestep_bytes": 8 * n,
        "bytes_per_launch": GOL_STEPS_PER_LAUNCH * 3 * n // 8,
        "state_bytes": 8 * n + 36,           # input + output + weights moved per e2e step
        "cpu_seconds": 12.0,
        "learning": False,
    }


def _inject_case(net_obj, inject, sizes_of):
    """Applies a parity case's injections (tests/golden/configs.py) to a
    built network; delays go in through the delay callback at build time."""
    for key, arr in inject.items():
        if key[2] == "delays":
            continue
        if key[0] == "neuron":
            dst = net_obj.get_neuron_data(key[1], key[2], key[3]).to_np_array()
        else:
            dst = net_obj.get_weight_matrix(key[1], key[2]).to_np_array()
        dst.view(arr.dtype)[:] = arr


def _case_network(net, inject_fn, seed):
    """(network dict with delay callbacks, injections, delays, sizes) of a
    parity case's network, for the bench's builds of the same configuration."""
    import numpy as np
    from tests.golden.cases import Case, callback_injections
    from tests.harness import case_sizes
    sizes = case_sizes(Case("bench", net, 1, seed))
    inj = inject_fn(np.random.default_rng(seed), sizes)
    delays = {k: v for k, v in inj.items() if k[2] == "delays"}
    net_dict, _, _, delay_arrays = callback_injections(net, delays)
    return net_dict, inj, delay_arrays, sizes


def _delay_callback(sg, delay_arrays):
    def delay_cb(ID, size, weights, delays):
        sg.IntArray(size, delays).to_np_array()[:] = delay_arrays[ID]
    if not hasattr(sg, "_delay_weight_callbacks"):
        sg._delay_weight_callbacks = {}
    sg.create_delay_weight_callback("golden_delay", delay_cb)


def iz_plastic_workload():
    """Large plastic Izhikevich network: three 256x256 Izhikevich layers with STDP on the convergent
    connection, a 4096x4096 subset projection and a 5 Hz Poisson drive."""
    from tests.golden import configs
    n = configs.C2_SIDE ** 2
    net = configs.c2_net(device_drive=11)
    net_dict, inj, delay_arrays, sizes = _case_network(net, configs.c2_inject, 221)

    def inject(net_obj):
        _inject_case(net_obj, inj, sizes)

    def result(net_obj):
        return net_obj.get_neuron_data("s", "L3", "output").to_np_array()

    conv, div, one, sub = n * 81, n, n, 4096 * 4096
    activate = conv + div + one + sub
    return {
        "name": "iz_plastic",
        "desc": "3x 256x256 Izhikevich (80% RS / 20% FS), L1->L2 convergent 9x9 STDP, "
                "L2->L3 divergent 3x3 stride 2, L3->L1 one-to-one, L2->L3 subset 4096x4096, "
                "delays U{0..3}, 5 Hz Poisson drive of value 20 generated on the device",
        "net": net_dict, "inject": inject, "result": result,
        "prepare": lambda sg: _delay_callback(sg, delay_arrays),
        "timesteps": 1000,
        "units_per_timestep": activate + conv,          # activator visits + updater visits
        "unit": "synapse-updates/s",
        "dtype": "f32",
        # algorithmic bytes per launch of each profiled kernel group
        # algorithmic bytes per launch of each profiled kernel group, the
        # per-synapse and per-neuron figures of the reference's data:
        # activator 32 B (w, stp r, stp w, delay, short and long trace r+w),
        # updater 40 B (w, presyn, wd, stp r/w, each read and written),
        # neuron 124 B
        "group_bytes": {"izhikevich.activate.subset": 32 * sub,
                        "izhikevich.learn.convergent": 40 * conv,
                        "izhikevich.activate.convergent": 32 * conv,
                        "izhikevich.activate.divergent": 32 * div,
                        "izhikevich.activate.one to one": 32 * one,
                        "izhikevich.update": 124 * 3 * n},
        "bytes_per_timestep": 32 * activate + 40 * conv + 3 * n * 124,
        # what this design moves: the subset connection never learns, so its
        # activator reads the product w * (R * w_stp), fixed during a run,
        # instead of the three arrays, and every activator here reads its
        # delays from a byte copy (21 and 29 B per synapse)
        "moved_bytes": {"izhikevich.activate.subset": 21 * sub,
                        "izhikevich.activate.convergent": 29 * conv},
        "state_bytes": None,                            # taken from the run report
        "cpu_seconds": 15.0,
        "learning": True,
    }


def iz_c0_workload():
    """The 32x32 plain Izhikevich network (no plasticity): relay input driven
    at 10 Hz on the device, convergent 5x5 wrap excitatory, recurrent fully
    connected inhibitory at 20% density, delays U{0..3}."""
    from tests.golden import configs
    net = configs.c0_net()
    net["structures"][0]["layers"][0]["init config"] = {"type": "poisson", "rate": 10,
                                                         "value": 1.0, "seed": 12}
    net_dict, inj, delay_arrays, sizes = _case_network(net, configs.c0_inject, 201)
    n = 32 * 32

    def inject(net_obj):
        _inject_case(net_obj, inj, sizes)

    def result(net_obj):
        return net_obj.get_neuron_data("s", "iz", "output").to_np_array()

    conv, fc = n * 25, n * n
    return {
        "name": "iz_c0",
        "desc": "32x32 relay (10 Hz Poisson drive generated on the device) -> 32x32 Izhikevich "
                "regular spiking, convergent 5x5 wrap U(0,0.5), recurrent fully connected 20% "
                "density U(0,0.2), delays U{0..3}, no plasticity",
        "net": net_dict, "inject": inject, "result": result,
        "prepare": lambda sg: _delay_callback(sg, delay_arrays),
        "timesteps": 1000,
        "units_per_timestep": conv + fc,
        "unit": "synapse-updates/s",
        "dtype": "f32",
        "group_bytes": {"izhikevich.activate.fully connected": 32 * fc,
                        "izhikevich.activate.convergent": 28 * conv,    # FLOAT source: no delay read
                        "izhikevich.update": 124 * n},
        "bytes_per_timestep": 32 * fc + 28 * conv + 124 * n,
        # the recurrent connection never learns: w * (R * w_stp) in one
        # array, delays as bytes
        "moved_bytes": {"izhikevich.activate.fully connected": 21 * fc},
        "l2_note": "34 MB per timestep: L2-resident within a bench step; flushed between steps",
        "state_bytes": None,
        "cpu_seconds": 10.0,
        "learning": False,
    }


def spnet_sparse_workload(side=256):
    """spnet (Izhikevich's polychronization model) with sparse connections: a
    256x256 excitatory layer with recurrent STDP over a 15x15 field, a 128x128
    inhibitory layer, half of every field's weights zero and compacted away,
    distance delays within the excitatory layer (1 step between the layers),
    a 5 Hz Poisson drive."""
    import numpy as np
    n = side * side

    def layer(name, rows, params, drive=False):
        d = {"name": name, "neural model": "spnet", "rows": rows, "columns": rows, "params": params}
        if drive:
            d["init config"] = {"type": "poisson", "rate": 5, "value": 20, "seed": 31}
        return d

    def weights(mx, seed):
        return {"type": "random", "min weight": 0.01, "max weight": mx, "fraction": 0.5, "seed": seed}
    net = {"structures": [{"name": "s", "type": "parallel", "layers": [
        layer("exc", side, "regular", drive=True), layer("inh", side // 2, "fast")]}],
        "connections": [
            {"name": "ee", "from layer": "exc", "to layer": "exc", "type": "convergent", "sparse": True,
             "opcode": "add", "plastic": True, "max weight": 10.0,
             "arborized config": {"field size": 15, "wrap": True}, "weight config": weights(6.0, 41)},
            {"name": "ei", "from layer": "exc", "to layer": "inh", "type": "convergent", "sparse": True,
             "opcode": "add", "plastic": False, "myelinated": True, "delay": 1,
             "arborized config": {"field size": 9, "stride": 2, "wrap": True},
             "weight config": weights(8.0, 42)},
            {"name": "ie", "from layer": "inh", "to layer": "exc", "type": "divergent", "sparse": True,
             "opcode": "sub", "plastic": False, "myelinated": True, "delay": 1,
             "arborized config": {"field size": 9, "stride": 2, "wrap": True},
             "weight config": weights(4.0, 43)}]}
    wl = {}

    def inject(net_obj):
        # synapses kept by the compaction: the nonzero compacted weights
        counts = {c: int(np.count_nonzero(net_obj.get_weight_matrix(c, "weights").to_np_array()))
                  for c in ("ee", "ei", "ie")}
        wl["synapses"] = counts
        wl["units_per_timestep"] = sum(counts.values()) + counts["ee"]   # activations + STDP
        wl["bytes_per_launch"] = 28 * counts["ee"]
        # the profiled groups this line can name: the STDP kernel (weight,
        # presynaptic trace and weight derivative read and written, source
        # index) and the three activations (weight, delay, source index)
        wl["group_bytes"] = {"spnet.learn.sparse": 28 * counts["ee"],
                             "spnet.activate.sparse": 12 * sum(counts.values()) // 3}

    def result(net_obj):
        return net_obj.get_neuron_data("s", "exc", "output").to_np_array()

    wl.update({
        "name": "spnet_sparse",
        "desc": "spnet 256x256 excitatory (recurrent STDP, convergent 15x15 wrap) + 128x128 "
                "inhibitory (convergent / divergent 9x9 stride 2), sparse connections with half "
                "of each field zero, distance delays (1 step between layers), 5 Hz Poisson drive",
        "net": net, "inject": inject, "result": result,
        "timesteps": 1000,
        "units_per_timestep": None,                     # set from the compacted state
        "unit": "synapse-updates/s",
        "dtype": "f32",
        "kernel": "spnet.learn.sparse",
        "bytes_per_launch": None,                       # w, presyn trace, dw r+w, source index
        "bytes_per_timestep": None,
        "state_bytes": None,
        "cpu_seconds": 8.0,
        "learning": True,
    })
    return wl


def batched_workload():
    """Batched instances: 256 independent instances of the plain Izhikevich
    configuration, sides uniform in 16..128 (seed 3), advanced together."""
    return {
        "name": "batched",
        "desc": "256 Izhikevich instances (relay->Izhikevich convergent 5x5 wrap, recurrent "
                "fully connected 20% density U(0,0.2), delays U{0..3}, 10 Hz relay drive), "
                "sides U{16..128} seed 3, a/b/c/d within +-10% of regular spiking",
        "timesteps": 100,
        "unit": "instance-timesteps/s",
        "dtype": "f32",
        "kernel": "k_batch_step",
        "cpu_seconds": 15.0,
        "batched": True,
    }


def rate_workload():
    """Differentiable rate network: forward pass and hand-written adjoint."""
    return {
        "name": "rate_adjoint",
        "desc": "3 x 64x64 leaky-integrator rate layers (tau 10 ms learnable, dt 1 ms, sigmoid "
                "rate), convergent 5x5 N(0,0.1), readout 4096->10 N(0,0.1), batch 64 x 100 "
                "steps of N(0,1) input, MSE to U(0,1) targets (seed 4), checkpoint every 10",
        "unit": "sequence-timesteps/s",
        "dtype": "f32",
        "kernel": "k_rate_fused (forward pass: one launch for all timesteps; time per timestep)",
        "cpu_seconds": 12.0,
        "rate": True,
    }


RATE_CFG = dict(layers=3, rows=64, cols=64, field=5, outputs=10, batch=64, steps=100,
                checkpoint=10)


def rate_inputs(batch=64, seed=4):
    """Seeded inputs and parameters of the rate workload (float32 numpy)."""
    import numpy as np
    c = RATE_CFG
    N = c["rows"] * c["cols"]
    rng = np.random.default_rng(seed)
    return {"x": rng.normal(0, 1, (c["steps"], batch, N)).astype(np.float32),
            "weights": rng.normal(0, 0.1, (c["layers"] - 1, N, c["field"] ** 2)).astype(np.float32),
            "readout": rng.normal(0, 0.1, (c["outputs"], N)).astype(np.float32),
            "tau": np.full(c["layers"], 10.0, np.float32),
            "target": rng.uniform(0, 1, (batch, c["outputs"])).astype(np.float32)}


WORKLOADS = {"gol": gol_workload, "iz_plastic": iz_plastic_workload, "iz_c0": iz_c0_workload,
             "batched": batched_workload, "rate_adjoint": rate_workload,
             "spnet_sparse": spnet_sparse_workload}
# the configurations nested in the default line, and their child-run arguments
SUB_RECORDS = (("iz_c0", []), ("gol", []), ("batched", ["--steps", "3", "--warmup", "3"]),
               ("rate_adjoint", []))

# Sides of the instances timed one at a time (plain GPU path / reference CPU
# path); the per-timestep time is fitted as alpha + beta * (recurrent synapses)
# and summed over the batch's instances.
PLAIN_SAMPLE_SIDES = (16, 32, 48, 64, 80, 96)
CPU_SAMPLE_SIDES = (16, 24, 32, 48, 64)


def sample_network(side):
    """One instance of the batch as an ordinary network, for timing only:
    connections are myelinated (delay 0) since distance-based default delays
    exceed 31 on large layers; a step's work does not depend on delay values."""
    from synaptogenesis_gb300 import batching
    net = batching.plain_network(batching.instance(side, 1))[0]
    for c in net["connections"]:
        c["myelinated"] = True
    return net


def fit_batch_seconds(samples, instances):
    """Seconds per timestep of running ``instances`` one at a time, from
    (side, seconds per timestep) samples fitted as alpha + beta * side**4."""
    import numpy as np
    x = np.array([float(s) ** 4 for s, _ in samples])
    y = np.array([t for _, t in samples])
    A = np.stack([np.ones_like(x), x], axis=1)
    (alpha, beta), *_ = np.linalg.lstsq(A, y, rcond=None)
    alpha, beta = max(alpha, 0.0), max(beta, 0.0)
    return sum(alpha + beta * float(i["rows"] * i["cols"]) ** 2 for i in instances), alpha, beta


# ---------------------------------------------------------------------------
# Helpers
# ---------------------------------------------------------------------------
def measured_peak():
    try:
        with open(PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.rows = []
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def dist_setup():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def reduce_max(values, world):
    if world == 1:
        return values
    import torch
    import torch.distributed as dist
    t = torch.tensor(values, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------------------
# CPU baseline: the reference's own library (or the oracle port) timed on the
# host cores on a bounded sample of the workload.
# ---------------------------------------------------------------------------
def cpu_worker(args):
    """Runs in a child process with SYNGEN_LIB set; prints one JSON object."""
    wl = WORKLOADS[args.workload]()
    if wl.get("rate"):
        # FP64 restatement (numpy, one thread): forward + adjoint of a sample of
        # the batch, the same 100 steps
        from oracle import rate_adjoint as ra
        sample_b = 8
        p = rate_inputs(batch=sample_b)
        shape = dict(RATE_CFG, batch=sample_b, dt=1.0)
        t0 = time.perf_counter()
        reps = 0
        while True:
            ra.adjoint(shape, p["x"], p["weights"], p["readout"], p["tau"], p["target"])
            reps += 1
            if time.perf_counter() - t0 >= args.cpu_seconds:
                break
        dt = time.perf_counter() - t0
        print(json.dumps({"value": sample_b * RATE_CFG["steps"] * reps / dt, "seconds": dt,
                          "timesteps": RATE_CFG["steps"] * reps, "reps": reps,
                          "sample_batch": sample_b}))
        return
    from synaptogenesis_gb300 import syngen as sg
    sg.set_warnings(False)
    if wl.get("batched"):
        # the reference runs one network at a time: time sample instances
        from synaptogenesis_gb300 import batching
        env = sg.Environment({"modules": []})
        run_args = {"multithreaded": False, "worker threads": 0, "learning flag": False}
        budget = args.cpu_seconds / len(CPU_SAMPLE_SIDES)
        samples, total_steps, total_s = [], 0, 0.0
        for side in CPU_SAMPLE_SIDES:
            net = sg.Network(sample_network(side))
            net.build_state()
            t0 = time.perf_counter()
            net.run(env, dict(run_args, iterations=2))
            per = max((time.perf_counter() - t0) / 2, 1e-6)
            steps = max(2, int(budget / per))
            t0 = time.perf_counter()
            rep = net.run(env, dict(run_args, iterations=steps))
            dt = time.perf_counter() - t0
            assert rep.obj is not None, "reference run failed"
            samples.append((side, dt / steps))
            total_steps += steps
            total_s += dt
            del net
        insts = batching.batch_instances(256, 3)
        secs, alpha, beta = fit_batch_seconds(samples, insts)
        print(json.dumps({"value": len(insts) / secs, "seconds": total_s, "timesteps": total_steps,
                          "samples": samples, "alpha": alpha, "beta": beta}))
        return
    if wl.get("prepare"):
        wl["prepare"](sg)
    net = sg.Network(wl["net"])
    net.build_state()
    wl["inject"](net)
    env = sg.Environment({"modules": []})
    run_args = {"multithreaded": False, "worker threads": 0, "learning flag": wl["learning"]}
    t0 = time.perf_counter()
    net.run(env, dict(run_args, iterations=2))
    per = max((time.perf_counter() - t0) / 2, 1e-6)
    steps = max(2, int(args.cpu_seconds / per))
    if args.cpu_timesteps:
        steps = args.cpu_timesteps
    t0 = time.perf_counter()
    rep = net.run(env, dict(run_args, iterations=steps))
    dt = time.perf_counter() - t0
    assert rep.obj is not None, "reference run failed"
    print(json.dumps({"value": wl["units_per_timestep"] * steps / dt, "seconds": dt,
                      "timesteps": steps}))


def cpu_baseline(workload, seconds, timesteps=0):
    if WORKLOADS[workload]().get("rate"):
        env = dict(os.environ, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1",
                   MKL_NUM_THREADS="1")
        cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--cpu-worker", "--workload",
               workload, "--cpu-seconds", str(seconds)]
        r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=900)
        if r.returncode != 0:
            return {"value": None, "unit": "sequence-timesteps/s", "cores": 1, "kind": "port",
                    "sample": "failed: " + r.stderr[-300:]}
        out = json.loads(r.stdout.strip().splitlines()[-1])
        return {"value": out["value"], "unit": "sequence-timesteps/s", "cores": 1, "kind": "port",
                "sample": "FP64 numpy restatement (oracle/rate_adjoint.py; the reference has no "
                          "differentiable model), forward + adjoint of %d sequences x 100 steps, "
                          "%d repetitions in %.1f s, one thread"
                          % (out["sample_batch"], out["reps"], out["seconds"]),
                "timesteps": out["timesteps"], "seconds": out["seconds"]}
    from oracle import build_ref
    lib = build_ref.build()
    cores = os.cpu_count() or 1
    if lib is None:
        return {"value": None, "unit": WORKLOADS[workload]()["unit"], "cores": 0, "kind": "reference",
                "sample": "unavailable: reference sources absent"}
    env = dict(os.environ, SYNGEN_LIB=lib, OMP_NUM_THREADS=str(cores))
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--cpu-worker", "--workload", workload,
           "--cpu-seconds", str(seconds), "--cpu-timesteps", str(timesteps)]
    r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=900)
    if r.returncode != 0:
        return {"value": None, "unit": WORKLOADS[workload]()["unit"], "cores": cores,
                "kind": "reference", "sample": "failed: " + r.stderr[-300:]}
    out = json.loads(r.stdout.strip().splitlines()[-1])
    if "samples" in out:
        sample = ("reference library run one instance at a time (dense recurrent matrix), "
                  "sides %s timed for %d timesteps in all (%.1f s wall, OMP_NUM_THREADS=%d); "
                  "per-timestep time fitted as %.3g s + %.3g s * side^4 and summed over the "
                  "256 instances" % (list(CPU_SAMPLE_SIDES), out["timesteps"], out["seconds"],
                                     cores, out["alpha"], out["beta"]))
    else:
        sample = ("%d timesteps of the same workload, %.1f s wall, OMP_NUM_THREADS=%d"
                  % (out["timesteps"], out["seconds"], cores))
    return {"value": out["value"], "unit": WORKLOADS[workload]()["unit"], "cores": cores,
            "kind": "reference", "sample": sample,
            "timesteps": out["timesteps"], "seconds": out["seconds"]}


# ---------------------------------------------------------------------------
# GB300 arm
# ---------------------------------------------------------------------------
def run_gb300(args, rank, world, local):
    import torch
    from synaptogenesis_gb300 import syngen as sg
    sg.set_warnings(False)
    wl = WORKLOADS[args.workload]()
    T = args.timesteps or wl["timesteps"]
    if wl.get("prepare"):
        wl["prepare"](sg)
    net = sg.Network(wl["net"])
    net.build_state()
    wl["inject"](net)
    run_args = {"learning flag": wl["learning"], "graph steps": 16}

    # -- device-resident throughput ------------------------------------------
    eng = sg.Engine(net, None, run_args)
    stream = torch.cuda.ExternalStream(eng.stream)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        eng.step(T)
    rep0 = eng.report()
    launches0 = int(rep0.properties["kernel launches"])
    gpu_index = os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[0]
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler(gpu_index)
    evs = []
    t_wall0 = time.perf_counter()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.add_(1.0)                       # L2 flush, outside the events
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.step(T)
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    barrier(world)
    clk = clocks.stop()
    dev_ms = sum(a.elapsed_time(b) for a, b in evs)
    rep1 = eng.report()
    launches = int(rep1.properties["kernel launches"]) - launches0
    eng.close()

    # -- per-kernel timing of the dominant kernel (separate profiled pass) ----
    prof_steps = min(T, 400)
    with sg.Engine(net, None, dict(run_args, profile=True)) as peng:
        peng.step(prof_steps)
        prep = peng.report()
    kern = {p.properties["name"]: p.properties for p in prep.child_arrays.get("kernel times", [])}
    total_ms = sum(float(k["total ms"]) for k in kern.values()) or 1.0
    for name, k in sorted(kern.items(), key=lambda kv: -float(kv[1]["total ms"])):
        print("# %-36s groups %7s  mean %9.2f us  share %5.1f%%"
              % (name, k["groups"], float(k["mean us"]), 100.0 * float(k["total ms"]) / total_ms),
              file=sys.stderr)
    mean_us = profiled_us = None
    dominant = wl.get("kernel")
    if wl.get("group_bytes"):
        # the kernel group with the largest share of the profiled pass
        ranked = sorted(kern.items(), key=lambda kv: -float(kv[1]["total ms"]))
        named = [(n, k) for n, k in ranked if n in wl["group_bytes"]]
        if named:
            dominant = named[0][0]
            wl["bytes_per_launch"] = wl["group_bytes"][dominant]
            mean_us = profiled_us = float(named[0][1]["mean us"])
        wl["shares"] = {n: round(float(k["total ms"]) / total_ms, 4) for n, k in ranked}
    if wl.get("timestep_bytes"):
        # every timed launch but two format conversions per run is the
        # multi-step kernel: its mean duration from the timed region
        mean_us = dev_ms * 1000.0 / (T * args.steps) * wl["steps_per_launch"]
        adv = kern.get(wl.get("profile_group", ""))
        if adv and int(adv["launches"]) > 0:
            profiled_us = 1000.0 * float(adv["total ms"]) / int(adv["launches"])
    wl["dominant"] = dominant

    # -- end to end through the public API with host buffers ----------------
    env = sg.Environment({"modules": []})
    wl["result"](net)                                      # state now lives on the host
    state_bytes = wl["state_bytes"] or int(rep1.properties["state bytes"])
    e2e_steps = max(1, min(args.steps, 3))

    def e2e_step():
        rep = net.run(env, dict(run_args, iterations=T))      # H2D of the state, then T timesteps
        assert rep.obj is not None, sg.last_error()
        res = wl["result"](net)                               # D2H of the state
        _ = int(res.view("uint32")[0])

    for _ in range(max(1, min(args.warmup, 2))):              # untimed, like the device leg
        e2e_step()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = time.perf_counter() - t0

    secs = dev_ms / 1000.0
    dev_max, = reduce_max([secs], world)
    e2e_max, = reduce_max([e2e_s], world)
    units = wl["units_per_timestep"] * T * args.steps
    out = {
        "dev_s": dev_max, "units": units * world, "wall_s": t_wall, "launches": launches,
        "mean_us": mean_us, "profiled_us": profiled_us, "clocks": clk, "kernels": kern,
        "e2e_value": wl["units_per_timestep"] * T * e2e_steps * world / e2e_max,
        "e2e_steps": e2e_steps, "wl": wl, "T": T, "state_bytes": state_bytes,
    }
    return out


def run_batched(args, rank, world, local):
    """The batch of instances (this rank's shard) on one GPU, plus the plain
    layer-by-layer GPU path run one instance at a time on sample instances."""
    import torch
    from synaptogenesis_gb300 import batching
    from synaptogenesis_gb300 import syngen as sg
    sg.set_warnings(False)
    wl = WORKLOADS[args.workload]()
    T = args.timesteps or wl["timesteps"]
    all_insts = batching.batch_instances(256, 3)
    if args.instances:
        # a smaller case of the same kernel (profiling): the largest instances
        all_insts = sorted(all_insts, key=lambda i: -i["rows"] * i["cols"])[:args.instances]
    insts = [all_insts[i] for i in batching.shard_instances(all_insts, rank, world)]
    b = sg.Batch(insts)
    rep0 = b.report()
    props = rep0.properties
    tuning = [{k: c.properties[k] for k in ("tile rows", "tile colblocks", "ms per step")}
              for c in rep0.child_arrays.get("autotune", [])]
    stream = torch.cuda.ExternalStream(b.stream)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        b.step(T)
    launches0 = int(b.report().properties["kernel launches"])
    gpu_index = os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[0]
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler(gpu_index)
    evs = []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.add_(1.0)                       # L2 flush, outside the events
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.step(T)
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    dev_s = sum(a.elapsed_time(c) for a, c in evs) / 1000.0
    launches = int(b.report().properties["kernel launches"]) - launches0

    # end to end: step through the C-ABI, then read every instance's output
    # words into host memory
    e2e_steps = max(1, min(args.steps, 3))
    d2h = sum(i["rows"] * i["cols"] for i in insts) * 4
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        b.step(T)
        outs = [b.read(i, "output") for i in range(len(insts))]
        _ = int(outs[-1][0])
    e2e_s = time.perf_counter() - t0
    b.close()

    # plain GPU path, one instance at a time (rank 0)
    plain = None
    if rank == 0 and not args.no_plain:
        samples = []
        for side in PLAIN_SAMPLE_SIDES:
            net = sg.Network(sample_network(side))
            net.build_state()
            with sg.Engine(net, None, {"learning flag": False, "graph steps": 16}) as eng:
                pst = torch.cuda.ExternalStream(eng.stream)
                eng.step(32)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(pst)
                eng.step(64)
                e1.record(pst)
                torch.cuda.synchronize()
                samples.append((side, e0.elapsed_time(e1) / 1000.0 / 64))
            del net
        secs, alpha, beta = fit_batch_seconds(samples, all_insts)
        plain = {"value": len(all_insts) / secs, "unit": wl["unit"],
                 "sample": "layer-by-layer GPU path (dense recurrent matrix), one instance at a "
                           "time, sides %s x 64 timesteps each; per-timestep time fitted as "
                           "%.3g s + %.3g s * side^4 and summed over the 256 instances"
                           % (list(PLAIN_SAMPLE_SIDES), alpha, beta),
                 "samples_s_per_timestep": samples}

    dev_max, e2e_max = reduce_max([dev_s, e2e_s], world)
    n_total = len(all_insts) if world > 1 else len(insts)
    return {"dev_s": dev_max, "units": n_total * T * args.steps, "launches": launches,
            "mean_us": dev_s * 1e6 / (T * args.steps), "clocks": clk, "T": T,
            "e2e_value": n_total * T * e2e_steps / e2e_max, "e2e_steps": e2e_steps,
            "d2h": d2h, "props": props, "tuning": tuning, "plain": plain,
            "step_bytes": int(props["step bytes"]),
            "syn_per_timestep": int(props["fc synapses"]) + int(props["conv synapses"])}


def batched_line(args, world, r, wl, cb):
    peak, peak_kind = measured_peak()
    p = r["props"]
    # algorithmic bytes: the non-zero recurrent synapses (read 16, write 8),
    # the convergent synapses (read 12, write 8) and the neurons (24); the
    # kernel also moves the ELL padding and the idle lanes of partial groups
    algo_bytes = (int(p["fc synapses"]) * 24 + int(p["conv synapses"]) * 20
                  + int(p["neurons"]) * 24)
    achieved = algo_bytes / (r["mean_us"] * 1e-6) / 1e9
    traffic = None
    try:
        with open(TRAFFIC) as f:
            traffic = json.load(f).get(args.workload)
    except Exception:
        pass
    value = r["units"] / r["dev_s"]
    return {
        "metric": "instance-timesteps/s (batched)", "value": value, "unit": wl["unit"],
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * r["dev_s"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": wl["dtype"], "data": "synthetic (counter-based generator, seeds per instance)",
        "config": {"workload": wl["desc"], "timesteps_per_step": r["T"],
                   "ms_per_timestep": 1000.0 * r["dev_s"] / (args.steps * r["T"]),
                   "synapse_updates_per_s": r["syn_per_timestep"] * r["T"] * args.steps / r["dev_s"],
                   "recurrent_synapses": int(p["fc synapses"]), "ell_slots": int(p["fc slots"]),
                   "convergent_synapses": int(p["conv synapses"]),
                   "device_bytes": int(p["device bytes"]),
                   "tile": [int(p["tile rows"]), int(p["tile colblocks"])],
                   "grid": int(p["grid"]), "threads": int(p["threads"]),
                   "autotune_ms_per_timestep": r["tuning"],
                   "l2": "flushed between steps (256 MiB write outside the timed events); "
                         "per-step traffic ~%.0f GB >> L2" % (r["step_bytes"] / 1e9),
                   "parallelism": "instances sharded over ranks" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": wl["kernel"], "bytes_per_launch": algo_bytes,
                     "moved_bytes_per_launch": r["step_bytes"],
                     "mean_launch_us": r["mean_us"]},
        "plain_gpu_one_at_a_time": r["plain"],
        "cpu_baseline": cb,
        "e2e": {"value": r["e2e_value"], "unit": wl["unit"], "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": r["d2h"], "steps": r["e2e_steps"],
                "note": "inputs are generated on the device from the instance seeds; every "
                        "instance's output words are read back each step"},
        "clocks": r["clocks"],
        "gpu_launches": r["launches"],
    }


def run_rate(args, rank, world, local):
    """Forward + adjoint of the rate workload, device-resident and end to end
    through the torch.autograd wrapper with host tensors; also the forward
    alone and the same work run one sequence at a time."""
    import torch
    from synaptogenesis_gb300 import syngen as sg
    c = RATE_CFG
    net = sg.RateNetwork(**c)
    host = rate_inputs()
    dev = {k: torch.tensor(v, device="cuda") for k, v in host.items()}
    stream = torch.cuda.current_stream()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    def fwd_bwd(net_, d):
        loss, ws = net_._forward(d["x"], d["weights"], d["readout"], d["tau"], d["target"])
        net_._backward(ws, 1.0, d["x"], d["weights"], d["readout"], d["tau"], d["target"],
                       want_dx=False)
        return loss

    def timed(fn, reps):
        out = []
        for _ in range(reps):
            flush.add_(1.0)                       # L2 flush, outside the events
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            out.append((e0, e1))
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in out) / 1000.0

    for _ in range(args.warmup):
        fwd_bwd(net, dev)
    torch.cuda.synchronize()
    barrier(world)
    gpu_index = os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[0]
    clocks = ClockSampler(gpu_index)
    dev_s = timed(lambda: fwd_bwd(net, dev), args.steps)
    barrier(world)
    clk = clocks.stop()
    fwd_s = timed(lambda: net._forward(dev["x"], dev["weights"], dev["readout"], dev["tau"],
                                       dev["target"]), args.steps)

    # one sequence at a time (batch 1, 64 calls) for the same work
    one = sg.RateNetwork(**dict(c, batch=1))
    singles = [{"x": dev["x"][:, b:b + 1].contiguous(), "weights": dev["weights"],
                "readout": dev["readout"], "tau": dev["tau"],
                "target": dev["target"][b:b + 1].contiguous()} for b in range(c["batch"])]
    fwd_bwd(one, singles[0])
    one_s = timed(lambda: [fwd_bwd(one, d) for d in singles], 1)

    # end to end: host inputs and parameters in, loss and gradients out
    e2e_steps = max(1, min(args.steps, 3))
    h2d = sum(v.nbytes for v in host.values())
    pinned = {k: torch.from_numpy(v).pin_memory() for k, v in host.items()}
    for _ in range(max(1, min(args.warmup, 2))):              # untimed, like the device leg
        t = {k: v.to("cuda", non_blocking=True) for k, v in pinned.items()}
        for k in ("weights", "readout", "tau"):
            t[k].requires_grad_(True)
        net.loss(t["x"], t["weights"], t["readout"], t["tau"], t["target"]).backward()
        torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        t = {k: v.to("cuda", non_blocking=True) for k, v in pinned.items()}
        for k in ("weights", "readout", "tau"):
            t[k].requires_grad_(True)
        loss = net.loss(t["x"], t["weights"], t["readout"], t["tau"], t["target"])
        loss.backward()
        grads = [t[k].grad.cpu() for k in ("weights", "readout", "tau")] + [loss.detach().cpu()]
    e2e_s = time.perf_counter() - t0
    d2h = sum(g.numel() * 4 for g in grads)

    per_step = c["batch"] * c["steps"]
    dev_max, e2e_max = reduce_max([dev_s, e2e_s], world)
    S = c["layers"] * c["batch"] * c["rows"] * c["cols"]
    N = c["rows"] * c["cols"]
    fwd_bytes = 16 * S + 4 * c["batch"] * N + 4 * ((c["layers"] - 1) * N * c["field"] ** 2
                                                   + c["outputs"] * N)
    return {"dev_s": dev_max, "units": per_step * args.steps * world, "clocks": clk,
            "fwd_s": fwd_s, "one_s": one_s, "e2e_value": per_step * e2e_steps * world / e2e_max,
            "e2e_steps": e2e_steps, "h2d": h2d, "d2h": d2h,
            "fwd_us_per_timestep": fwd_s * 1e6 / (args.steps * c["steps"]),
            "fwd_bytes_per_timestep": fwd_bytes, "loss": float(loss.detach())}


def rate_line(args, world, r, wl, cb):
    peak, peak_kind = measured_peak()
    c = RATE_CFG
    per_step = c["batch"] * c["steps"]
    achieved = r["fwd_bytes_per_timestep"] / (r["fwd_us_per_timestep"] * 1e-6) / 1e9
    # kernel launches per forward + adjoint: forward = weight transpose, the
    # multi-step forward kernel, outputs, loss; backward = weight transpose,
    # dloss/dy, per segment the multi-step recompute, dW and its accumulation,
    # dR and its accumulation, dtau partials, per timestep an adjoint step,
    # and the dtau total
    nseg = -(-c["steps"] // c["checkpoint"])
    launches = 4 + (2 + 6 * nseg + c["steps"] + 1)
    return {
        "metric": "sequence-timesteps/s (rate forward + adjoint)",
        "value": r["units"] / r["dev_s"], "unit": wl["unit"], "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * r["dev_s"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": wl["dtype"],
        "data": "synthetic (seeded numpy)",
        "config": {"workload": wl["desc"], "sequence_timesteps_per_step": per_step,
                   "forward_only_sequence_timesteps_per_s": per_step * args.steps / r["fwd_s"],
                   "one_sequence_at_a_time_sequence_timesteps_per_s": per_step / r["one_s"],
                   "loss": r["loss"],
                   "l2": "flushed between steps (256 MiB write outside the timed events); the "
                         "state (3 MB per timestep) is L2-resident within a step",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "peak_kind": peak_kind,
                     "kernel": wl["kernel"], "bytes_per_launch": r["fwd_bytes_per_timestep"],
                     "mean_launch_us": r["fwd_us_per_timestep"]},
        "cpu_baseline": cb,
        "e2e": {"value": r["e2e_value"], "unit": wl["unit"], "h2d_bytes_per_step": r["h2d"],
                "d2h_bytes_per_step": r["d2h"], "steps": r["e2e_steps"],
                "note": "torch.autograd path: pinned host inputs and parameters copied in, "
                        "loss.backward(), gradients and loss copied out"},
        "clocks": r["clocks"],
        "gpu_launches": launches * args.steps,
    }


def sub_records(args):
    """The other measured configurations, each from a child run of this
    script on the same GPU (one JSON line each)."""
    out = {}
    for name, extra in SUB_RECORDS:
        cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--workload", name,
               "--steps", str(min(args.steps, 10)), "--warmup", str(max(3, min(args.warmup, 3)))]
        cmd += extra
        if args.no_cpu_baseline:
            cmd.append("--no-cpu-baseline")
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=1200)
            lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
            if r.returncode != 0 or not lines:
                out[name] = {"failed": (r.stderr or r.stdout)[-400:]}
                continue
            out[name] = json.loads(lines[-1])
        except Exception as e:                              # noqa: BLE001
            out[name] = {"failed": repr(e)[:400]}
    return out


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="iz_plastic", choices=sorted(WORKLOADS))
    p.add_argument("--no-sub", action="store_true",
                   help="default workload: leave out the nested configurations")
    p.add_argument("--timesteps", type=int, default=0, help="timesteps per bench step")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--instances", type=int, default=0,
                   help="batched workload: only the N largest instances (profiling case)")
    p.add_argument("--no-plain", action="store_true",
                   help="batched workload: skip the one-instance-at-a-time plain GPU timing")
    p.add_argument("--cpu-worker", action="store_true", help=argparse.SUPPRESS)
    p.add_argument("--cpu-seconds", type=float, default=0.0, help=argparse.SUPPRESS)
    p.add_argument("--cpu-timesteps", type=int, default=0, help=argparse.SUPPRESS)
    args = p.parse_args()
    if args.cpu_worker:
        cpu_worker(args)
        return

    rank, world, local = dist_setup()
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = os.environ.get("CUDA_VISIBLE_DEVICES",
                                                            ",".join(str(i) for i in range(world))
                                                            ).split(",")[local]
        import torch.distributed as dist
        dist.init_process_group("gloo")
    wl = WORKLOADS[args.workload]()
    metric = ("instance-timesteps/s (batched)" if wl.get("batched")
              else "sequence-timesteps/s (rate forward + adjoint)" if wl.get("rate")
              else "synapse-updates/s (%s)" % wl["name"])

    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import build_ref
        if not wl.get("rate") and build_ref.build() is None:
            print(json.dumps({"impl": "reference", "unavailable": "reference sources absent"}))
            return
        # each bench step: a bounded sample of the workload on all host cores
        per_step_s = max(1.0, 60.0 / max(1, args.steps + args.warmup))
        cb = cpu_baseline(args.workload, per_step_s * (args.steps + args.warmup))
        if cb["value"] is None:
            print(json.dumps({"impl": "reference", "unavailable": cb["sample"]}))
            return
        ts_per_step = max(1, cb["timesteps"] // max(1, args.steps + args.warmup))
        ms_per_step = 1000.0 * cb["seconds"] / max(1, args.steps + args.warmup)
        line = {"metric": metric, "value": cb["value"], "unit": wl["unit"], "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": wl["dtype"], "data": "synthetic", "impl": "reference",
                "config": {"workload": wl["desc"], "timesteps_per_step": ts_per_step,
                           "host_threads": cb["cores"]},
                "cpu_baseline": dict(cb),
                "e2e": {"value": cb["value"], "unit": wl["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if wl.get("rate"):
        r = run_rate(args, rank, world, local)
        if rank != 0:
            return
        cb = None if args.no_cpu_baseline else cpu_baseline(args.workload, wl["cpu_seconds"])
        print(json.dumps(rate_line(args, world, r, wl, cb)))
        return
    if wl.get("batched"):
        r = run_batched(args, rank, world, local)
        if rank != 0:
            return
        cb = None if args.no_cpu_baseline else cpu_baseline(args.workload, wl["cpu_seconds"])
        print(json.dumps(batched_line(args, world, r, wl, cb)))
        return

    r = run_gb300(args, rank, world, local)
    if rank != 0:
        return
    wl = r["wl"]                 # as built: workloads may size themselves from their state
    peak, peak_kind = measured_peak()
    achieved = None
    if r["mean_us"]:
        achieved = wl["bytes_per_launch"] / (r["mean_us"] * 1e-6) / 1e9
    traffic = None
    try:
        with open(TRAFFIC) as f:
            traffic = json.load(f).get(args.workload)
    except Exception:
        pass
    cb = None
    if not args.no_cpu_baseline:
        cb = cpu_baseline(args.workload, wl["cpu_seconds"])
    value = r["units"] / r["dev_s"]
    ms_per_timestep = 1000.0 * r["dev_s"] / (args.steps * r["T"])
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None,
                "traffic": traffic.get(wl["dominant"]) if isinstance(traffic, dict) else traffic,
                "peak_kind": peak_kind,
                "kernel": wl["dominant"], "bytes_per_launch": wl.get("bytes_per_launch"),
                "mean_launch_us": r["mean_us"],
                "profiled_launch_us": r["profiled_us"],
                "word_layout_bytes_per_timestep": wl.get("word_layout_timestep_bytes")}
    if wl.get("shares"):
        roofline["profiled_shares"] = wl["shares"]
    moved = (wl.get("moved_bytes") or {}).get(wl["dominant"])
    if moved and r["mean_us"]:
        # the bytes this design's kernel must move (fewer than the
        # reference's data holds), over the same launch time
        roofline["moved_bytes_per_launch"] = moved
        roofline["moved_frac"] = moved / (r["mean_us"] * 1e-6) / 1e9 / peak
    if wl.get("bytes_per_timestep"):
        # the whole timestep: every kernel's algorithmic bytes over the
        # device time per timestep
        step_gbs = wl["bytes_per_timestep"] / (ms_per_timestep * 1e-3) / 1e9
        roofline["step"] = {"bytes_per_timestep": wl["bytes_per_timestep"],
                            "ms_per_timestep": ms_per_timestep, "achieved": step_gbs,
                            "frac": step_gbs / peak}
    line = {
        "metric": metric, "value": value, "unit": wl["unit"], "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * r["dev_s"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": wl["dtype"], "data": "synthetic",
        "config": {"workload": wl["desc"], "timesteps_per_step": r["T"],
                   "ms_per_timestep": ms_per_timestep,
                   "l2": wl.get("l2_note", "flushed between steps (256 MiB write outside the "
                                           "timed events)"),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": roofline,
        "cpu_baseline": cb,
        "e2e": {"value": r["e2e_value"], "unit": wl["unit"],
                "h2d_bytes_per_step": r["state_bytes"], "d2h_bytes_per_step": r["state_bytes"],
                "steps": r["e2e_steps"]},
        "clocks": r["clocks"],
        "gpu_launches": r["launches"],
    }
    if world == 1 and args.workload == "iz_plastic" and not args.no_sub:
        line["configs"] = sub_records(args)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
