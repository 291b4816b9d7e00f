"""The N > 1 path (independent replicas) with two gloo ranks on the CPU."""

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from bldfm_gb300.replicas import shard


def test_shard_covers_every_case_once():
    for n in (0, 1, 7, 16, 513):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                a, b = shard(n, r, world)
                assert 0 <= a <= b <= n
                seen.extend(range(a, b))
            assert seen == list(range(n))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_q):
    import torch.distributed as dist

    from bldfm_gb300.replicas import max_time_ms, solve_sharded
    from oracle import bldfm_oracle as O

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cases = []
    for j in range(5):
        z, p = O.vertical_profiles(8, 5.0, (2.0 + j, -1.0), ustar=0.3, mol=-40.0)
        cases.append(dict(srf_flx=np.zeros((24, 32)), z=z, profiles=p, domain=(64.0, 48.0), levels=8,
                          modes=(32, 24), meas_pt=(20.0, 20.0), footprint=True, precision="double"))

    def solve(sub):
        return [O.steady_state_transport_solver(**kw)[2] for kw in sub]

    res = solve_sharded(cases, solve)
    t = max_time_ms(10.0 * (rank + 1))
    if rank == 0:
        ref = solve(cases)
        out_q.put((len(res), all(np.array_equal(a, b) for a, b in zip(res, ref)), t))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas_gather_in_case_order():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    n, same, t = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert n == 5 and same
    assert t == 20.0  # slowest rank's time
