"""The replica harness of bench.py (enjaparticles_gb300.replicas) with two gloo
ranks on the CPU: barrier, max and sum over ranks."""
import os
import socket
import time

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from enjaparticles_gb300.replicas import Replicas
    r = Replicas(backend="gloo")
    time.sleep(0.2 * rank)  # rank 1 arrives late
    t0 = time.perf_counter()
    r.barrier()
    waited = time.perf_counter() - t0
    out.put((rank, r.max(1.0 + rank), r.sum(10.0 * (rank + 1)), waited))
    r.close()


def test_two_gloo_ranks_max_sum_barrier():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(k, world, port, q)) for k in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, sm, waited in res:
        assert mx == 2.0 and sm == 30.0
    assert res[0][3] >= 0.1  # rank 0 waited for rank 1 at the barrier


def test_single_process_is_identity():
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE"):
        os.environ.pop(k, None)
    from enjaparticles_gb300.replicas import Replicas
    r = Replicas()
    assert r.world == 1 and r.max(3.5) == 3.5 and r.sum(2.0) == 2.0
    r.barrier()
    r.close()
