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


def _natgrad_data():
    import numpy as np
    rng = np.random.default_rng(17)
    rows = rng.normal(size=(10, 7))
    w = rng.random(10) + 0.1
    e = rng.normal(size=10)
    return rows, w, e


def _natgrad_single(rows, w, e, step, error):
    """The reference's conjugate gradient (observer.py:576-675) over all samples in one process."""
    import numpy as np
    W = w.sum()
    E = (w * e).sum() / W
    delta = (w[:, None] * rows).sum(axis=0) / W
    param = np.sqrt(w / W)
    Dm = (rows - delta) * param[:, None]
    En = (e - E) * param
    b = Dm.T @ En
    x = np.zeros_like(b)
    r = b - Dm.T @ (Dm @ x)
    p, rr, t = r, r @ r, 0
    while t != step and not (error != 0.0 and error**2 > rr / (b @ b)):
        Dp = Dm @ p
        alpha = rr / (Dp @ Dp)
        x = x + alpha * p
        r = r - alpha * (Dm.T @ Dp)
        new = r @ r
        p = r + (new / rr) * p
        rr = new
        t += 1
    return 2 * x


class _FakeEngine:
    """The engine calls the Observer makes, over this rank's hole rows held in host memory."""

    def __init__(self, rows, w, e):
        import numpy as np
        self.rows, self.w, self.e = rows, w, e
        self.np = np

    def keep_holes(self, enable=True):
        pass

    def reset_observer(self):
        pass

    def read_observer(self, with_gradient=True):
        np = self.np
        scalars = np.array([len(self.w), self.w.sum(), (self.w**2).sum(), 0.0, (self.w * self.e).sum(), 0.0, 0.0, 0.0])
        delta = (self.w[:, None] * self.rows).sum(axis=0)
        edelta = ((self.w * self.e)[:, None] * self.rows).sum(axis=0)
        return scalars, delta, edelta

    def holes_gemv(self, x, transpose=False):
        return self.rows.T @ x if transpose else self.rows @ x

    def holes_gram(self):
        return self.rows @ self.rows.T


class _FakeOwner:
    site_number = 1
    _active_observer = None

    def unflatten(self, flat):
        return flat


def _natgrad_worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from tnsp_gb300.sampling import Observer
    from test_multirank import _FakeEngine, _FakeOwner, _natgrad_data
    rows, w, e = _natgrad_data()
    mine = slice(rank, None, world)
    out = []
    for step, error in [(3, 0.0), (50, 1e-6)]:
        obs = Observer(_FakeOwner(), enable_natural_gradient=True)
        obs.__enter__()
        obs._bind(_FakeEngine(rows[mine], w[mine], e[mine]))
        obs._samples_w = w[mine].tolist()
        obs._samples_e = e[mine].tolist()
        obs.__exit__(None, None, None)
        out.append(obs.natural_gradient_by_conjugate_gradient(step, error).tolist())
    q.put((rank, out))
    dist.destroy_process_group()


def test_two_rank_natural_gradient_equals_one_process():
    """Samples split over two gloo ranks: the drop-in Observer's conjugate gradient (its D^T u and
    |Dp|^2 summed over the ranks) gives the one-process solution over all samples."""
    import numpy as np
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_natgrad_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    rows, w, e = _natgrad_data()
    for k, (step, error) in enumerate([(3, 0.0), (50, 1e-6)]):
        want = _natgrad_single(rows, w, e, step, error)
        for rank, results in out:
            np.testing.assert_allclose(results[k], want, rtol=1e-10, atol=1e-12)


def _observer_set_worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import numpy as np
    from tnsp_gb300.sampling import Observer
    from test_multirank import _FakeEngine, _FakeOwner3, _observer_set_data
    confs, w, e, sets = _observer_set_data()
    mine = slice(rank, None, world)
    obs = Observer(_FakeOwner3(), observer_set=sets, enable_energy=True)
    obs.__enter__()
    obs._bind(_FakeEngine(np.zeros((len(w[mine]), 1)), w[mine], e[mine]))
    obs._observe_set(confs[mine], w[mine])
    obs.__exit__(None, None, None)
    res = obs.result
    q.put((rank, {n: {str(k): v for k, v in d.items()} for n, d in res.items()}, obs.whole_result))
    dist.destroy_process_group()


class _FakeOwner3:
    L1 = L2 = 3
    site_number = 9
    _active_observer = None


def _observer_set_data():
    import numpy as np
    rng = np.random.default_rng(31)
    confs = (rng.random((12, 3, 3)) < 0.5).astype(np.int64)
    w = rng.random(12) + 0.2
    e = rng.normal(size=12)
    sz = {(0,): [((0,), 0.5)], (1,): [((1,), -0.5)]}
    szsz = {(a, b): [((a, b), 0.25 * (1 - 2 * a) * (1 - 2 * b))] for a in (0, 1) for b in (0, 1)}
    sets = {"Sz": {((1, 1, 0),): sz, ((2, 0, 0),): sz}, "SzSz": {((0, 0, 0), (2, 2, 0)): szsz}}
    return confs, w, e, sets


def test_two_rank_observer_set_equals_one_process():
    """Diagonal observer-set accumulators split over two gloo ranks are summed like the reference's
    MPI reduction: results equal the one-process ones."""
    import numpy as np
    from tnsp_gb300.sampling import Observer
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_observer_set_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    confs, w, e, sets = _observer_set_data()
    one = Observer(_FakeOwner3(), observer_set=sets, enable_energy=True)
    one.__enter__()
    one._bind(_FakeEngine(np.zeros((len(w), 1)), w, e))
    one._observe_set(confs, w)
    one.__exit__(None, None, None)
    want = {n: {str(k): v for k, v in d.items()} for n, d in one.result.items()}
    for rank, res, whole in out:
        for n in want:
            for k in want[n]:
                np.testing.assert_allclose(res[n][k], want[n][k], rtol=1e-12)
            np.testing.assert_allclose(whole[n], one.whole_result[n], rtol=1e-12)
        np.testing.assert_allclose(whole["energy"], one.whole_result["energy"], rtol=1e-12)


def test_pseudo_inverse_natural_gradient_in_one_process():
    """The drop-in pseudo-inverse natural gradient (single-process form of observer.py:697-907) on rows
    held by a stand-in engine: against the same equation evaluated directly, and, with a tiny
    regulariser, x / 2 solves the least-squares equations D^T D (x / 2) = D^T (E - <E>).  (T = D D^T
    always has the weight vector as a null vector, so some regularisation is required.)"""
    import numpy as np
    sys.path.insert(0, ROOT)
    from tnsp_gb300.sampling import Observer
    rows, w, e = _natgrad_data()
    for r_pinv, a_pinv in [(1e-6, 1e-9), (1e-3, 1e-12), (1e-9, 0.0)]:
        obs = Observer(_FakeOwner(), enable_natural_gradient=True)
        obs.__enter__()
        obs._bind(_FakeEngine(rows, w, e))
        obs._samples_w = w.tolist()
        obs._samples_e = e.tolist()
        obs.__exit__(None, None, None)
        x = obs.natural_gradient_by_direct_pseudo_inverse(r_pinv, a_pinv)
        W = w.sum()
        delta = (w[:, None] * rows).sum(axis=0) / W
        D = rows - delta
        E = e - (w * e).sum() / W
        L, U = np.linalg.eigh(D @ D.T)
        num = r_pinv * L.max() + a_pinv
        Linv = np.array([0.0 if l <= 0 else 1.0 / (l * (1 + (num / l)**6)) for l in L])
        want = 2 * D.T @ (U @ (Linv * (U.T @ E)))
        np.testing.assert_allclose(x, want, rtol=1e-8, atol=1e-12)
        if r_pinv == 1e-9:
            np.testing.assert_allclose(D.T @ (D @ (x / 2)), D.T @ E, rtol=1e-6, atol=1e-9)
