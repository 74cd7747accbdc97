"""Served fits: a continuous-batching request loop on one GPU context.

Requests (one cube each, its grid on the device or on the host) arrive from any
thread through ``FitServer.submit``, which returns a ``concurrent.futures.Future``.
A dispatcher thread groups waiting requests into batches of one size class
(large cubes, by their estimated device footprint, are batched apart from the
rest, so a small request never waits inside a batch for a large cube): at most
``max_batch`` cubes, at most ``max_wait_s`` after the oldest waiting request
arrived.  Admission is by device memory: a batch is submitted only while the
estimated bytes of every batch in flight plus its own stay within ``hbm_budget``
(a request that alone exceeds the budget is rejected).  Batches go to the
context's worker with ``rp_batch_submit``; the worker keeps up to three of them
in flight on the device at once (each in a slot of its own), so a batch that
arrives while others run starts at once and overlaps them.  A completion thread
polls the tickets and resolves each request's future as soon as its batch is
done, in whatever order batches finish.  A cube's charges do not depend on the
batch it was served in (the batched fit is bitwise independent of its neighbours
and of the streams and slot it runs on).

No reference counterpart: repeat.py is a one-shot program.  The serving workload
(Poisson arrivals from the batch distribution) is measured by ``bench.py``.
"""
from __future__ import annotations

import collections
import queue
import threading
import time
from concurrent.futures import Future

from . import _lib

GRAM_LANES = 4  # streams of a batch's normal equations, each with its own scratch


def footprint(cube) -> tuple[int, int]:
    """(fixed, scratch) estimated device bytes of a cube in a batch: its grid-sized
    arrays (grid values, kept indices, centred ESP), and, bounded by the whole grid,
    the scratch of its normal equations (fixed-point digits of every atom row,
    reciprocal rows), which a batch holds once per gram stream, not per cube."""
    nx, ny, nz = (int(v) for v in cube.n_grid)
    npts = nx * ny * nz
    N = int(cube.n_atoms)
    return 20 * npts, 8 * (N + 1) * npts + 8 * ny * nz * N * int(cube.kmax)


def device_bytes(cube) -> int:
    """Estimated device bytes of a cube fitted alone."""
    fixed, scratch = footprint(cube)
    return fixed + scratch


def batch_bytes(cubes) -> int:
    """Estimated device bytes of a batch: every cube's fixed arrays plus the largest
    scratch once per gram stream in use."""
    fp = [footprint(c) for c in cubes]
    if not fp:
        return 0
    return sum(f for f, _ in fp) + min(GRAM_LANES, len(fp)) * max(s for _, s in fp)


class _Request:
    __slots__ = ("cube", "V_dev", "future", "t_arrive", "t_done", "bytes")

    def __init__(self, cube, V_dev):
        self.cube, self.V_dev = cube, V_dev
        self.future = Future()
        self.t_arrive = time.perf_counter()
        self.t_done = None
        self.bytes = device_bytes(cube)


class FitServer:
    """Continuous-batching fit server on ``ctx`` (a ``pyrepeat_gb300.fit.Context``).

    ``large_bytes``: requests whose estimated footprint exceeds it form batches of
    their own, of at most ``max_large_batch`` cubes."""

    def __init__(self, ctx, max_batch: int = 64, max_wait_s: float = 0.002, hbm_budget: float = 150e9,
                 precision: int = _lib.PREC_MIXED, large_bytes: float = 8e9, max_large_batch: int = 1):
        self.ctx = ctx
        self.max_batch = int(max_batch)
        self.max_wait_s = float(max_wait_s)
        self.hbm_budget = float(hbm_budget)
        self.precision = precision
        self.large_bytes = float(large_bytes)
        self.max_large_batch = int(max_large_batch)
        self._in: queue.Queue = queue.Queue()
        self._submitted: queue.Queue = queue.Queue()
        self._closed = False
        self.latencies: list[float] = []  # seconds, arrival to charges on the host, per request
        self.batch_sizes: list[int] = []
        self.large_latencies: list[float] = []   # the same, large requests only
        self.small_latencies: list[float] = []   # the same, every other request
        self.max_in_flight = 0            # most batches in flight at once (submitted, not retired)
        self._lock = threading.Lock()
        self._cv = threading.Condition()
        self._inflight_bytes = 0
        self._inflight = 0
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
    def _large(self, r) -> bool:
        return r.bytes > self.large_bytes

    def _dispatch(self):
        pend = {False: collections.deque(), True: collections.deque()}  # waiting requests by class
        stopping = False
        while True:
            if not pend[False] and not pend[True]:
                if stopping:
                    break
                r = self._in.get()
                if r is None:
                    break
                pend[self._large(r)].append(r)
            # the class of the oldest waiting request fills a batch until its wait bound
            cls = min((c for c in (False, True) if pend[c]), key=lambda c: pend[c][0].t_arrive)
            limit = self.max_large_batch if cls else self.max_batch
            deadline = pend[cls][0].t_arrive + self.max_wait_s
            while len(pend[cls]) < limit and not stopping:
                timeout = deadline - time.perf_counter()
                try:
                    r = self._in.get(timeout=timeout) if timeout > 0 else self._in.get_nowait()
                except queue.Empty:
                    break
                if r is None:
                    stopping = True
                    break
                pend[self._large(r)].append(r)
            batch = [pend[cls].popleft()]
            while pend[cls] and len(batch) < limit and batch_bytes(
                    [x.cube for x in batch] + [pend[cls][0].cube]) <= self.hbm_budget:
                batch.append(pend[cls].popleft())
            need = batch_bytes([x.cube for x in batch])
            with self._cv:  # admission: bytes of every batch in flight stay within the budget
                while self._inflight and self._inflight_bytes + need > self.hbm_budget:
                    self._cv.wait()
                self._inflight_bytes += need
                self._inflight += 1
                self.max_in_flight = max(self.max_in_flight, self._inflight)
            self._submit(batch, need)
        self._submitted.put(None)

    def _release(self, need):
        with self._cv:
            self._inflight_bytes -= need
            self._inflight -= 1
            self._cv.notify_all()

    def _submit(self, batch, need):
        cubes = [r.cube for r in batch]
        V_dev = [r.V_dev for r in batch]
        try:
            pb = self.ctx.batch_submit(cubes, self.precision, V_dev if any(v is not None for v in V_dev) else None)
        except Exception as e:  # noqa: BLE001 - handed to every request of the batch
            for r in batch:
                r.future.set_exception(e)
            self._release(need)
            return
        self._submitted.put((pb, batch, need))

    def _finish(self, pb, batch, need):
        try:
            q, M, info = pb.result()
        except Exception as e:  # noqa: BLE001
            for r in batch:
                r.future.set_exception(e)
            self._release(need)
            return
        now = time.perf_counter()
        with self._lock:
            self.batch_sizes.append(len(batch))
            for r in batch:
                r.t_done = now
                self.latencies.append(now - r.t_arrive)
                (self.large_latencies if self._large(r) else self.small_latencies).append(now - r.t_arrive)
        self._release(need)
        for r, qi in zip(batch, q):
            r.future.set_result(qi.copy())

    def _complete(self):
        outstanding = []
        ended = False
        while True:
            # new batches (block only when nothing is in flight)
            while True:
                try:
                    item = self._submitted.get(block=not outstanding and not ended)
                except queue.Empty:
                    break
                if item is None:
                    ended = True
                    break
                outstanding.append(item)
                if not self._submitted.qsize():
                    break
            # retire every finished batch, in the order they finish
            still = []
            for item in outstanding:
                try:
                    done = item[0].poll()
                except Exception:  # noqa: BLE001 - result() raises it to the requests
                    done = True
                if done:
                    self._finish(*item)
                else:
                    still.append(item)
            progressed = len(still) != len(outstanding)
            outstanding = still
            if ended and not outstanding:
                return
            if outstanding and not progressed:
                time.sleep(0.0002)
