"""CPU tests of the batched runner's host side: the numpy counter generator
against an independent big-integer restatement, the instance generator, the
plain-network builder, argument validation at the C-ABI, and the sharding of
instances over ranks (two gloo processes, no data exchange in the path)."""
import os

import numpy as np
import pytest

from synaptogenesis_gb300 import batching

MASK = (1 << 64) - 1


def ref_bits(seed, stream, index):
    z = (seed * 0x9E3779B97F4A7C15 + stream * 0xD1B54A32D192ED03 + index) & MASK
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
    return z ^ (z >> 31)


@pytest.mark.parametrize("seed,stream", [(0, 1), (3, 5), (2**63 + 12345, 2), (300007, 4)])
def test_counter_generator_matches_restatement(seed, stream):
    idx = np.array([0, 1, 2, 77, 2**31 + 5, 2**40 + 3], dtype=np.uint64)
    got = batching.counter_bits(seed, stream, idx)
    want = [ref_bits(seed, stream, int(i)) for i in idx]
    assert [int(x) for x in got] == want
    u = batching.counter_uniform(seed, stream, idx)
    assert u.dtype == np.float32
    assert [float(x) for x in u] == [float(np.float32((w >> 40) / 16777216.0)) for w in want]
    d = batching.counter_below(seed, stream, idx, 4)
    assert [int(x) for x in d] == [(w >> 32) % 4 for w in want]


def test_batch_instances_configuration():
    insts = batching.batch_instances(256, 3)
    assert len(insts) == 256
    sides = np.array([x["rows"] for x in insts])
    assert sides.min() >= 16 and sides.max() <= 128 and len(set(sides)) > 50
    assert len({x["seed"] for x in insts}) == 256
    for k in "abcd":
        ratio = np.array([x[k] for x in insts]) / batching.REGULAR[k]
        assert ratio.min() >= 0.9 - 1e-6 and ratio.max() <= 1.1 + 1e-6
    assert batching.batch_instances(256, 3) == insts


def test_plain_network_injections():
    inst = batching.instance(10, 42)
    net, inj, inputs = batching.plain_network(inst)
    n = 100
    w = inj[("matrix", "c_rec", "weights")]
    assert w.shape == (n * n,) and w.dtype == np.float32
    density = (w != 0).mean()
    assert 0.15 < density < 0.25
    assert w.max() < 0.2 and w.min() >= 0.0
    d = inj[("matrix", "c_rec", "delays")]
    assert set(np.unique(d)) <= {0, 1, 2, 3}
    assert inj[("matrix", "c_in", "weights")].shape == (n * 25,)
    x = np.stack([inputs(t) for t in range(200)])
    assert set(np.unique(x)) <= {0.0, 1.0} and 0.005 < x.mean() < 0.015


def test_batch_rejects_invalid_instances():
    from synaptogenesis_gb300 import syngen
    bad = [dict(batching.instance(4, 1), conv_field=9),
           dict(batching.instance(8, 1), fc_max_delay=32),
           dict(batching.instance(8, 1), input_rate=1.5),
           dict(batching.instance(8, 1), rows=0)]
    for spec in bad:
        with pytest.raises(RuntimeError, match="batch: instance 0"):
            syngen.Batch([spec])
    with pytest.raises(RuntimeError, match="no instances"):
        syngen.Batch([])


def test_shard_instances_single_rank():
    insts = batching.batch_instances(64, 9)
    assert batching.shard_instances(insts, 0, 1) == list(range(64))
    with pytest.raises(ValueError):
        batching.shard_instances(insts, 2, 2)


def _shard_worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    insts = batching.batch_instances(256, 3)
    mine = batching.shard_instances(insts, rank, world)
    parts = [None] * world
    dist.all_gather_object(parts, mine)
    if rank == 0:
        q.put(parts)
    dist.destroy_process_group()


def test_shard_instances_two_gloo_ranks():
    import multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    parts = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    a, b = map(set, parts)
    assert not (a & b) and a | b == set(range(256))
    insts = batching.batch_instances(256, 3)
    la = sum(batching.instance_cost(insts[i]) for i in a)
    lb = sum(batching.instance_cost(insts[i]) for i in b)
    assert abs(la - lb) / (la + lb) < 0.01
