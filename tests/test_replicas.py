"""Multi-rank bookkeeping on CPU (gloo, world size 2): each rank evaluates
its own shard of candidates with the CPU oracle; the slowest rank's time and
the aggregate throughput are computed as the benchmark does; a rank that
leaves between steps is detected by the other through the store."""
import os
import socket
import time

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _env(rank, world, port):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})


def _shard_worker(rank, world, port, out):
    _env(rank, world, port)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from lensed_gb300 import quadrature, replicas, workloads
    from oracle.oracle import Oracle

    r, w, _, dist = replicas.init("gloo", timeout_s=60)
    s = workloads.small()
    cand = workloads.draw_candidates(s, 2, seed=replicas.candidate_seed(r))
    o = Oracle(s.plugins, s.width, s.height, quadrature.rule(s.rule), image=s.image, weight=s.weight, threads=1)
    dist.barrier()
    t0 = time.perf_counter()
    ll = o.loglike(cand)
    dt = time.perf_counter() - t0
    dist.barrier()
    tmax = replicas.max_over_ranks(dt, dist)
    out[r] = (ll.tolist(), dt, tmax, replicas.aggregate(len(cand), tmax, w))
    dist.destroy_process_group()


def test_two_rank_shards_and_aggregate():
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_shard_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    from lensed_gb300 import quadrature, replicas, workloads
    from oracle.oracle import Oracle

    s = workloads.small()
    o = Oracle(s.plugins, s.width, s.height, quadrature.rule(s.rule), image=s.image, weight=s.weight, threads=1)
    for r in range(world):
        want = o.loglike(workloads.draw_candidates(s, 2, seed=replicas.candidate_seed(r)))
        assert np.array_equal(np.array(res[r][0]), want)  # shards are independent
    tmax = max(res[r][1] for r in range(world))
    for r in range(world):
        assert res[r][2] == pytest.approx(tmax)
        assert res[r][3] == pytest.approx(world * 2 / tmax)
    assert not np.array_equal(res[0][0], res[1][0])  # different candidates per rank


def _dying_worker(rank, world, port, out):
    _env(rank, world, port)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from lensed_gb300 import replicas
    import torch.distributed as dist

    replicas.init("gloo", timeout_s=20)
    store = dist.distributed_c10d._get_default_store()
    hb = replicas.Heartbeat(store, rank, world, timeout_s=3)
    hb.beat(0)
    out[f"missing0_{rank}"] = hb.missing(0)
    if rank == 1:
        out["left"] = True
        os._exit(0)  # leaves between steps, nothing in flight
    hb.beat(1)
    out["missing1_0"] = hb.missing(1)


def test_rank_that_leaves_is_detected_before_the_next_step():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_dying_worker, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=60)
        for p in procs:
            if p.is_alive():
                p.kill()
        res = dict(out)
    assert res["missing0_0"] == [] and res["missing0_1"] == []
    assert res.get("left")
    assert res["missing1_0"] == [1]
