"""Sharding independent particles across ranks (gloo, world_size 2 on CPU):
the shards cover every particle once and the gathered end states equal a
single-process run (the integrator being the oracle here, the multi-GPU path
being the same host logic around the device integrator)."""
import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from assist_gb300.shard import gather_states, shard_indices


def test_shards_partition():
    lengths = np.exp(np.random.default_rng(0).uniform(np.log(30), np.log(3652), 1001))
    for world in (1, 2, 3, 8):
        parts = [shard_indices(lengths, r, world) for r in range(world)]
        allidx = np.sort(np.concatenate(parts))
        assert np.array_equal(allidx, np.arange(lengths.size))
        loads = [lengths[p].sum() for p in parts]
        assert max(loads) - min(loads) <= lengths.max() + 1e-9


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, paths, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from assist_gb300 import synth
    from tests.oracle_py import Oracle
    pl, ast = paths
    system = synth.SolarSystem(4242)
    pop = synth.population(system, "mix", 12, seed=9, t0=8000.0, log_len=(10.0, 100.0))
    idx = shard_indices(pop.t_end - pop.t0, rank, world)
    o = Oracle(pl, ast)
    st = o.integrate_batch(pop.t0[idx], pop.t_end[idx], pop.state[idx], threads=1)
    got = [None] * world
    dist.all_gather_object(got, (idx, st))
    if rank == 0:
        q.put(gather_states(got, 12))
    dist.destroy_process_group()


def test_gloo_two_ranks_gather(golden_paths):
    from assist_gb300 import synth
    from tests.oracle_py import Oracle
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, golden_paths, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    system = synth.SolarSystem(4242)
    pop = synth.population(system, "mix", 12, seed=9, t0=8000.0, log_len=(10.0, 100.0))
    ref = Oracle(*golden_paths).integrate_batch(pop.t0, pop.t_end, pop.state, threads=1)
    assert np.array_equal(res, ref)
