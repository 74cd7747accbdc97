"""The serving layer: asynchronous batches (rp_batch_submit / poll / wait) and the
continuous-batching FitServer.

CPU: the dispatcher's batching rules (batch size, wait bound, size classes, HBM
admission across the batches in flight, rejection, completion in any order) against
a fake context.  GPU: requests served from two threads in mixed batches give exactly
the charges of each cube fitted alone; a small batch submitted behind a large one
finishes first while both are in flight; the C-ABI tickets retire as documented."""
import threading
import time

import numpy as np
import pytest

from conftest import load_golden
from pyrepeat_gb300 import serve


class _FakeCube:
    def __init__(self, n_atoms, n_grid=(10, 10, 10), kmax=7):
        self.n_atoms = n_atoms
        self.n_grid = np.array(n_grid)
        self.kmax = kmax


class _FakePending:
    def __init__(self, cubes, gate=None):
        self.cubes = cubes
        self.gate = gate   # a threading.Event: the batch is done once it is set

    def poll(self):
        return self.gate is None or self.gate.is_set()

    def result(self):
        return [np.full(c.n_atoms, float(c.n_atoms)) for c in self.cubes], np.zeros(len(self.cubes)), None


class _FakeCtx:
    """Records the batches the server submits; results are available at once, or once
    the gate given for a batch is set."""

    def __init__(self, gates=None):
        self.batches = []
        self.gates = gates or {}

    def batch_submit(self, cubes, precision, V_dev):
        self.batches.append([c.n_atoms for c in cubes])
        return _FakePending(cubes, self.gates.get(len(self.batches) - 1))


def test_batches_respect_size_and_admission():
    ctx = _FakeCtx()
    one = serve.device_bytes(_FakeCube(5))
    srv = serve.FitServer(ctx, max_batch=4, max_wait_s=0.2, hbm_budget=3.5 * one)
    futs = [srv.submit(_FakeCube(5)) for _ in range(7)]
    srv.close()
    assert [f.result()[0] for f in futs] == [5.0] * 7
    assert sum(len(b) for b in ctx.batches) == 7
    assert max(len(b) for b in ctx.batches) <= 3           # admission: 3 cubes fit the budget, not 4
    assert len(srv.latencies) == 7 and srv.batch_sizes == [len(b) for b in ctx.batches]


def test_oversize_request_is_rejected():
    ctx = _FakeCtx()
    srv = serve.FitServer(ctx, hbm_budget=1e3)
    f = srv.submit(_FakeCube(50))
    with pytest.raises(MemoryError):
        f.result(timeout=5)
    srv.close()
    assert ctx.batches == []


def test_wait_bound_closes_a_partial_batch():
    ctx = _FakeCtx()
    srv = serve.FitServer(ctx, max_batch=64, max_wait_s=0.01)
    f1 = srv.submit(_FakeCube(3))
    assert f1.result(timeout=5)[0] == 3.0                  # served without a full batch
    f2 = srv.submit(_FakeCube(4))
    assert f2.result(timeout=5)[0] == 4.0
    srv.close()
    assert ctx.batches == [[3], [4]]


class _FailingCtx:
    def batch_submit(self, cubes, precision, V_dev):
        raise RuntimeError("device lost")


class _FailingResultCtx(_FakeCtx):
    def batch_submit(self, cubes, precision, V_dev):
        super().batch_submit(cubes, precision, V_dev)

        class P:
            def poll(self_inner):
                return True

            def result(self_inner):
                raise RuntimeError("batch failed")
        return P()


def test_errors_reach_every_request_of_the_batch():
    for ctx, msg in ((_FailingCtx(), "device lost"), (_FailingResultCtx(), "batch failed")):
        srv = serve.FitServer(ctx, max_batch=4, max_wait_s=0.05)
        futs = [srv.submit(_FakeCube(3)) for _ in range(3)]
        srv.close()
        for f in futs:
            with pytest.raises(RuntimeError, match=msg):
                f.result(timeout=5)
        assert srv.latencies == []


def test_large_requests_are_batched_apart():
    """A large cube forms a batch of its own: the small requests around it are not
    held inside its batch."""
    ctx = _FakeCtx()
    small = _FakeCube(5)
    big = _FakeCube(40, n_grid=(60, 60, 60))
    srv = serve.FitServer(ctx, max_batch=8, max_wait_s=0.05, large_bytes=serve.device_bytes(small) * 10)
    futs = [srv.submit(c) for c in (small, big, small, small)]
    srv.close()
    assert [f.result()[0] for f in futs] == [5.0, 40.0, 5.0, 5.0]
    assert sorted(ctx.batches) == [[5, 5, 5], [40]]
    assert len(srv.large_latencies) == 1


def test_admission_counts_batches_in_flight():
    """A batch whose bytes, added to the batches still in flight, exceed the budget waits
    until one of them retires; batches that fit run side by side."""
    one = serve.batch_bytes([_FakeCube(5)])
    gates = {0: threading.Event(), 1: threading.Event()}
    ctx = _FakeCtx(gates=gates)
    srv = serve.FitServer(ctx, max_batch=1, max_wait_s=0.0, hbm_budget=2.5 * one)
    f = [srv.submit(_FakeCube(5)) for _ in range(3)]
    time.sleep(0.05)
    assert len(ctx.batches) == 2 and not any(x.done() for x in f)   # two fit side by side, a third waits
    gates[1].set()
    assert f[1].result(timeout=5)[0] == 5.0 and f[2].result(timeout=5)[0] == 5.0
    assert not f[0].done()                         # batches retire as they finish, in any order
    gates[0].set()
    assert f[0].result(timeout=5)[0] == 5.0
    srv.close()
    assert srv.max_in_flight == 2


def test_closed_server_refuses_requests():
    srv = serve.FitServer(_FakeCtx())
    srv.close()
    with pytest.raises(RuntimeError):
        srv.submit(_FakeCube(3))


@pytest.mark.gpu
def test_served_fits_equal_fits_alone(gpu_ctx):
    """Alone vs mixed: each request's charges equal the cube fitted alone, bitwise."""
    from pyrepeat_gb300 import _lib
    names = ("water24", "tricmini", "mofmini")
    alone = {n: gpu_ctx.fit_host(load_golden(n)[0], precision=_lib.PREC_MIXED).charges for n in names}
    srv = serve.FitServer(gpu_ctx, max_batch=8, max_wait_s=0.003)
    results = {}

    def client(k):
        rng = np.random.default_rng(k)
        for t in range(12):
            name = names[int(rng.integers(3))]
            results[(k, t)] = (name, srv.submit(load_golden(name)[0]))
            time.sleep(float(rng.uniform(0, 0.002)))

    th = [threading.Thread(target=client, args=(k,)) for k in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    srv.close()
    for (name, fut) in results.values():
        assert np.array_equal(fut.result(timeout=60), alone[name]), name
    assert sum(srv.batch_sizes) == 24 and len(srv.latencies) == 24


@pytest.mark.gpu
def test_small_batch_overtakes_a_large_one(gpu_ctx):
    """Continuous batching on the device: a small batch submitted right behind a large
    cube's batch runs beside it (its own slot, higher stream priority) and finishes first;
    both results equal the fits alone, bitwise."""
    from pyrepeat_gb300 import _lib, synth
    large = synth.make_batch_item(90001, large=True, ctx=gpu_ctx)
    small, _ = load_golden("water24")
    alone_large = gpu_ctx.fit_batch([large], _lib.PREC_MIXED, V_dev=[large.V_dev])[0][0].copy()
    alone_small = gpu_ctx.fit_host(small, precision=_lib.PREC_MIXED).charges
    order = []
    for rep in range(2):   # the first round sizes both slots' buffers
        pl = gpu_ctx.batch_submit([large], _lib.PREC_MIXED, V_dev=[large.V_dev])
        ps = gpu_ctx.batch_submit([small], _lib.PREC_MIXED)
        done = {}
        t0 = time.perf_counter()
        while len(done) < 2:
            for name, pb in (("large", pl), ("small", ps)):
                if name not in done and pb.poll():
                    done[name] = time.perf_counter() - t0
            assert time.perf_counter() - t0 < 120
            time.sleep(0.0002)
        order.append(done)
        assert np.array_equal(pl.result()[0][0], alone_large)
        assert np.array_equal(ps.result()[0][0], alone_small)
    assert order[1]["small"] < order[1]["large"], order


@pytest.mark.gpu
def test_batch_tickets(gpu_ctx):
    import ctypes
    from pyrepeat_gb300 import _lib
    cube, _ = load_golden("water24")
    pb1 = gpu_ctx.batch_submit([cube], _lib.PREC_MIXED)
    pb2 = gpu_ctx.batch_submit([cube, cube], _lib.PREC_MIXED)
    q2, M2, _ = pb2.result()
    q1, M1, _ = pb1.result()
    assert np.array_equal(q1[0], q2[0]) and np.array_equal(q2[0], q2[1]) and M1[0] == M2[1]
    done, st = ctypes.c_int(), ctypes.c_int()
    # a retired ticket is unknown
    assert gpu_ctx.lib.rp_batch_poll(gpu_ctx.ptr, pb1.ticket, ctypes.byref(done), ctypes.byref(st)) == _lib.RP_E_ARG
