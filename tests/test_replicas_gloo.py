"""Multi-rank host path on CPU (gloo, world_size 2): AOI sharding, max-over-ranks timing
and the whole-job throughput the bench reports for N > 1 replicas."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update({'RANK': str(rank), 'WORLD_SIZE': str(world), 'LOCAL_RANK': str(rank),
                       'MASTER_ADDR': '127.0.0.1', 'MASTER_PORT': str(port)})
    from vissatsatellitestereo_gb300 import replicas
    r, w, _ = replicas.init('gloo')
    costs = [5.0, 1.0, 3.0, 3.0, 2.0, 8.0, 1.0]
    mine = replicas.shard_balanced(costs, w)[r]
    units = sum(costs[i] for i in mine)
    elapsed = 1.0 + r                   # rank 1 is the slow one
    replicas.barrier()
    out[r] = (mine, replicas.max_over_ranks(elapsed), replicas.job_throughput(units, elapsed))
    replicas.finish()


@pytest.mark.timeout(120)
def test_two_gloo_ranks():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    shards = [res[0][0], res[1][0]]
    assert sorted(shards[0] + shards[1]) == list(range(7))          # every AOI once
    assert not set(shards[0]) & set(shards[1])
    assert res[0][1] == res[1][1] == 2.0                             # slowest rank's time
    assert res[0][2] == res[1][2] == pytest.approx(23.0 / 2.0)      # all units / max time


def test_balanced_sharding_single_process():
    from vissatsatellitestereo_gb300 import replicas
    shards = replicas.shard_balanced([4, 4, 4, 4, 1, 1], 2)
    loads = [sum([4, 4, 4, 4, 1, 1][i] for i in s) for s in shards]
    assert loads == [9, 9]
    assert replicas.shard_balanced([1, 2, 3], 1) == [[0, 1, 2]]
    assert replicas.job_throughput(10.0, 2.0) == 5.0                 # no process group: local
