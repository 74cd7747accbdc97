"""Served fits: a micro-batching request loop on one GPU context.

Requests (one cube each, its grid on the device or on the host) arrive from any
thread through ``FitServer.submit``, which returns a ``concurrent.futures.Future``.
A dispatcher thread groups waiting requests into batches: at most ``max_batch``
cubes, at most ``max_wait_s`` after the oldest waiting request arrived, and an
estimated device footprint within ``hbm_budget`` bytes (admission control: a
request that does not fit waits for the next batch; one that alone exceeds the
budget is rejected).  Each batch goes to the context's worker with
``rp_batch_submit``, so the next batch is assembled while the device runs the
current one; a completion thread resolves every request's future when its batch is
done.  A cube's charges do not depend on the batch it was served in (the batched
fit is bitwise independent of its neighbours and of the stream a cube runs on).

No reference counterpart: repeat.py is a one-shot program.  The serving workload
(Poisson arrivals from the batch distribution) is measured by ``bench.py
--workload serve``.
"""
from __future__ import annotations

import collections
import queue
import threading
import time
from concurrent.futures import Future

from . import _lib


def device_bytes(cube) -> int:
    """Estimated device bytes a cube adds to a batch: its grid-sized arrays (grid values,
    kept indices, centred ESP) and, bounded by the whole grid, the per-stream scratch of
    its normal equations (fixed-point digits of every atom row, reciprocal rows)."""
    nx, ny, nz = (int(v) for v in cube.n_grid)
    npts = nx * ny * nz
    N = int(cube.n_atoms)
    fixed = 20 * npts
    scratch = 8 * (N + 1) * npts + 8 * ny * nz * N * int(cube.kmax)
    return fixed + scratch


class _Request:
    __slots__ = ("cube", "V_dev", "future", "t_arrive", "t_done", "bytes")

    def __init__(self, cube, V_dev):
        self.cube, self.V_dev = cube, V_dev
        self.future = Future()
        self.t_arrive = time.perf_counter()
        self.t_done = None
        self.bytes = device_bytes(cube)


class FitServer:
    """Micro-batching fit server on ``ctx`` (a ``pyrepeat_gb300.fit.Context``)."""

    def __init__(self, ctx, max_batch: int = 64, max_wait_s: float = 0.002, hbm_budget: float = 150e9,
                 precision: int = _lib.PREC_MIXED):
        self.ctx = ctx
        self.max_batch = int(max_batch)
        self.max_wait_s = float(max_wait_s)
        self.hbm_budget = float(hbm_budget)
        self.precision = precision
        self._in: queue.Queue = queue.Queue()
        self._submitted: queue.Queue = queue.Queue()
        self._closed = False
        self.latencies: list[float] = []  # seconds, arrival to charges on the host, per request
        self.batch_sizes: list[int] = []
        self._lock = threading.Lock()
        self._dispatcher = threading.Thread(target=self._dispatch, name="fit-dispatch", daemon=True)
        self._completer = threading.Thread(target=self._complete, name="fit-complete", daemon=True)
        self._dispatcher.start()
        self._completer.start()

    # ------------------------------------------------------------------ API
    def submit(self, cube, V_dev=None) -> Future:
        """Queue one fit; the future's result is the cube's charges (numpy array)."""
        if self._closed:
            raise RuntimeError("FitServer is closed")
        r = _Request(cube, V_dev)
        if r.bytes > self.hbm_budget:
            r.future.set_exception(MemoryError(
                f"cube needs ~{r.bytes / 1e9:.1f} GB of device memory, over the server's budget "
                f"{self.hbm_budget / 1e9:.1f} GB"))
            return r.future
        self._in.put(r)
        return r.future

    def close(self, wait: bool = True):
        """Stop accepting requests; with wait, serve the queued ones first."""
        self._closed = True
        self._in.put(None)
        if wait:
            self._dispatcher.join()
            self._completer.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------------ threads
    def _dispatch(self):
        carry: collections.deque = collections.deque()  # admitted-later requests, oldest first
        stopping = False
        while True:
            if carry:
                first = carry.popleft()
            else:
                if stopping:
                    break
                first = self._in.get()
                if first is None:
                    break
            batch, used = [first], first.bytes
            deadline = first.t_arrive + self.max_wait_s
            while len(batch) < self.max_batch:
                if carry:
                    r = carry.popleft()
                else:
                    timeout = deadline - time.perf_counter()
                    try:
                        r = self._in.get(timeout=max(timeout, 0.0)) if timeout > 0 else self._in.get_nowait()
                    except queue.Empty:
                        break
                    if r is None:
                        stopping = True
                        break
                if used + r.bytes > self.hbm_budget:
                    carry.appendleft(r)  # admission: waits for the next batch
                    break
                batch.append(r)
                used += r.bytes
            self._submit(batch)
        self._submitted.put(None)

    def _submit(self, batch):
        cubes = [r.cube for r in batch]
        V_dev = [r.V_dev for r in batch]
        try:
            pb = self.ctx.batch_submit(cubes, self.precision, V_dev if any(v is not None for v in V_dev) else None)
        except Exception as e:  # noqa: BLE001 - handed to every request of the batch
            for r in batch:
                r.future.set_exception(e)
            return
        self._submitted.put((pb, batch))

    def _complete(self):
        while True:
            item = self._submitted.get()
            if item is None:
                return
            pb, batch = item
            try:
                q, M, info = pb.result()
            except Exception as e:  # noqa: BLE001
                for r in batch:
                    r.future.set_exception(e)
                continue
            now = time.perf_counter()
            with self._lock:
                self.batch_sizes.append(len(batch))
                for r, qi in zip(batch, q):
                    r.t_done = now
                    self.latencies.append(now - r.t_arrive)
            for r, qi in zip(batch, q):
                r.future.set_result(qi.copy())
