"""The N>1 path of bench.py: replicas, no data-path collective; only the timing is reduced
(max over ranks) and the samples are summed.  Two gloo ranks on CPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.reduce_over_ranks(dist, 1.0 + rank, "max")
    n = bench.reduce_over_ranks(dist, 456.0, "sum")
    q.put((rank, t, n))
    dist.destroy_process_group()


def test_two_rank_timing_and_sample_reduction():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, n in out:
        assert t == 2.0  # the slowest rank's time
        assert n == 912.0  # samples of both replicas


def _observer_worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import numpy as np
    from tnsp_gb300.sampling import allreduce_sum, default_seeds
    scalars = np.arange(8, dtype=np.float64) * (rank + 1)
    delta = np.full(5, 0.5 + rank)
    edelta = np.full(5, -1.0 * rank)
    s, d, e = allreduce_sum([scalars, delta, edelta])
    q.put((rank, s.tolist(), d.tolist(), e.tolist(), default_seeds(3, 100).tolist()))
    dist.destroy_process_group()


def test_two_rank_observer_reduction_and_seeds():
    """The drop-in Observer sums its accumulators over the ranks (the reference's MPI Allreduce in
    Observer.__exit__) and every rank draws distinct default chain seeds."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_observer_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, s, d, e, seeds in out:
        assert s == [3.0 * k for k in range(8)]
        assert d == [2.0] * 5
        assert e == [-1.0] * 5
    assert out[0][4] == [100, 101, 102] and out[1][4] == [103, 104, 105]


def test_single_process_reduction_is_identity():
    import numpy as np
    sys.path.insert(0, ROOT)
    from tnsp_gb300.sampling import allreduce_sum, default_seeds
    a = np.arange(4.0)
    (b,) = allreduce_sum([a])
    assert (a == b).all()
    assert default_seeds(2, 7).tolist() == [7, 8]
