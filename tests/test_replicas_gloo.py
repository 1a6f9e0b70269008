"""Multi-GPU runs are replicas (no collective on the data path): bench.py's
harness puts a barrier around the timed region and takes the slowest rank's
time.  This exercises that harness with two gloo ranks on the CPU, each rank
advancing its own replica of a small problem with the oracle."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import time

    import oracle as O

    import bench

    dist = bench.init_dist(world)
    ps = O.Space1D(0, 1, 50 + 10 * rank, 2)
    P = O.Problem(O.ADVECTION, ps, a=1.0)
    state = {"u": np.sin(2 * np.pi * ps.xpg)}

    def advance(n):
        state["u"] = P.ssprk3(state["u"], 1e-3, n)
        if rank == 1:
            time.sleep(0.2)  # the slow rank sets the job's time

    secs = bench.run_replicas(advance, 5, 2, lambda: None, dist)
    q.put((rank, secs, float(np.max(np.abs(state["u"])))))
    dist.destroy_process_group()


def test_replica_harness_takes_the_slowest_rank():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    secs = {r: s for r, s, _ in out}
    # both ranks report the same (maximum) time, at least the slow rank's sleep
    assert secs[0] == pytest.approx(secs[1])
    assert secs[0] >= 0.2
    assert all(abs(m - 1.0) < 1e-2 for _, _, m in out)
