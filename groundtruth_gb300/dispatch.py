"""Boards fanned out to worker processes, one per GPU (replicas: a board is solved whole on one device and
nothing crosses between workers), with the host-side failure handling of GroundTruth's compute server
(remote/worker.py:1-30: one job per worker process and a watchdog over it; solver/gpu.py:70-80: a failed device
run reported, not hidden).

Each worker is a spawned process that owns one device (``CUDA_VISIBLE_DEVICES`` is set before the job function is
unpickled) and talks to the dispatcher over its own pipe, so a worker that is killed while sending corrupts nothing
the others use.  The dispatcher hands every idle worker the next job and watches the busy ones:

* a worker that exits (a crash, a kill from outside) has its job handed to the next free worker and is replaced;
* a job that runs past ``timeout`` seconds has its worker killed (the process the dispatcher started, by its own
  handle), replaced, and the job handed on the same way;
* a job that goes that way ``attempts`` times is reported failed with ``WorkerLost``;
* a job whose function raises (``SolverError``, ``MemoryError``, ``ValueError``) is reported failed at once with the
  exception's text: it would fail the same way again.

A worker is only ever stopped between jobs or by killing its whole process, never with a device call of its own in
flight from another thread, so the device contexts of the surviving workers are not touched.
"""
from __future__ import annotations

import os
import pickle
import time
from collections import deque
from dataclasses import dataclass
from multiprocessing import connection
from typing import Any, Callable, Optional, Sequence

import multiprocessing as mp


class WorkerLost(RuntimeError):
    """A job's worker died or overran its time limit on every attempt."""


@dataclass
class Outcome:
    id: int                      # the job's index in the list given to map()
    ok: bool
    value: Any = None            # fn(payload) when ok
    error: Optional[str] = None  # "<ExceptionType>: <text>" when not ok
    attempts: int = 0            # workers the job was handed to
    worker: Optional[int] = None  # the slot of the worker that finished (or last held) it
    seconds: float = 0.0         # the finishing worker's time in fn


def _serve(conn, device, fn_bytes: bytes):
    """A worker's loop: receive (id, payload), run fn, send back (id, ok, pickled value or error, seconds); None
    ends it."""
    if device is not None:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(device)
    fn = pickle.loads(fn_bytes)
    while True:
        try:
            item = conn.recv()
        except EOFError:
            return
        if item is None:
            return
        jid, payload = item
        t0 = time.perf_counter()
        try:
            msg = (jid, True, pickle.dumps(fn(payload)), time.perf_counter() - t0)
        except Exception as e:          # noqa: BLE001 — reported to the dispatcher, which decides
            msg = (jid, False, f"{type(e).__name__}: {e}", time.perf_counter() - t0)
        conn.send(msg)


class Dispatcher:
    """``workers`` processes running ``fn`` (a module-level function, so that it pickles) on payloads.

    devices: the device of each worker (default: none set, the worker sees what the parent sees); timeout: seconds
    a job may run before its worker is killed (None: no limit); attempts: workers a job is handed to before it is
    reported lost."""

    def __init__(self, fn: Callable[[Any], Any], workers: int = 1, devices: Optional[Sequence] = None,
                 timeout: Optional[float] = None, attempts: int = 2):
        if workers < 1:
            raise ValueError("at least one worker")
        if devices is not None and len(devices) != workers:
            raise ValueError("one device per worker")
        if attempts < 1:
            raise ValueError("at least one attempt per job")
        self._fn = pickle.dumps(fn)
        self._ctx = mp.get_context("spawn")
        self.devices = list(devices) if devices is not None else [None] * workers
        self.timeout, self.attempts = timeout, attempts
        self.procs: list = [None] * workers
        self.conns: list = [None] * workers
        self.replaced = 0                # workers started again after a death or a kill
        for s in range(workers):
            self._start(s)

    def _start(self, slot: int):
        parent, child = self._ctx.Pipe(duplex=True)
        p = self._ctx.Process(target=_serve, args=(child, self.devices[slot], self._fn), daemon=True)
        p.start()
        child.close()
        self.procs[slot], self.conns[slot] = p, parent

    def _retire(self, slot: int):
        p = self.procs[slot]
        if p.is_alive():
            p.kill()
        p.join()
        self.conns[slot].close()
        return p.exitcode

    def map(self, payloads: Sequence) -> list:
        """Every payload through fn on the workers: an Outcome per payload, in the payloads' order."""
        n = len(payloads)
        out: list = [None] * n
        tries = [0] * n
        pending = deque(range(n))
        busy: dict = {}                  # slot -> (job, start time)
        while any(o is None for o in out):
            for s in range(len(self.procs)):
                if s in busy or not pending:
                    continue
                if not self.procs[s].is_alive():
                    self._retire(s)
                    self._start(s)
                    self.replaced += 1
                j = pending.popleft()
                tries[j] += 1
                self.conns[s].send((j, payloads[j]))
                busy[s] = (j, time.monotonic())
            if not busy:
                continue
            wait = None
            if self.timeout is not None:
                wait = max(0.0, min(t0 + self.timeout for _, t0 in busy.values()) - time.monotonic())
            ready = connection.wait([self.conns[s] for s in busy] + [self.procs[s].sentinel for s in busy], wait)
            now = time.monotonic()
            for s, (j, t0) in list(busy.items()):
                reason = None
                if self.conns[s] in ready:
                    try:
                        jid, ok, data, secs = self.conns[s].recv()
                    except (EOFError, OSError):
                        reason = "exited"
                    else:
                        del busy[s]
                        if out[jid] is None:
                            out[jid] = Outcome(jid, ok, pickle.loads(data) if ok else None, None if ok else data,
                                               tries[jid], s, secs)
                        continue
                elif self.procs[s].sentinel in ready or not self.procs[s].is_alive():
                    reason = "exited"
                elif self.timeout is not None and now - t0 >= self.timeout:
                    reason = f"timed out after {self.timeout:g} s"
                if reason is None:
                    continue
                del busy[s]
                code = self._retire(s)
                if reason == "exited":
                    reason = f"worker exited with code {code}"
                self._start(s)
                self.replaced += 1
                if out[j] is not None:
                    continue
                if tries[j] < self.attempts:
                    pending.appendleft(j)
                else:
                    out[j] = Outcome(j, False, None, f"WorkerLost: {reason} (attempt {tries[j]})", tries[j], s)
        return out

    def close(self):
        """Stop every worker between jobs; one that does not stop within a few seconds is killed."""
        for s, p in enumerate(self.procs):
            if p is None:
                continue
            if p.is_alive():
                try:
                    self.conns[s].send(None)
                except (BrokenPipeError, OSError):
                    pass
            p.join(5.0)
            self._retire(s)
        self.procs = [None] * len(self.procs)

    def __enter__(self) -> "Dispatcher":
        return self

    def __exit__(self, *exc):
        self.close()


def solve_board(arrays: dict) -> dict:
    """One board (``synth.Board.to_arrays``) solved whole on the worker's device: every net at every frequency of the
    board, in one batch (PlaneStack.solve per route and frequency, peec.py:2513, 2787).  Returns the frequencies and
    per (net, frequency) the loop impedance, the moment, the iterations and the final FP64 residual."""
    import numpy as np

    from . import stack as gs, synth
    board = synth.Board.from_arrays(arrays)
    st, routes = gs.from_board(board)
    sols = gs.solve_many(routes, board.freqs, tol=board.tol, restart=board.restart)
    return {"freqs": np.asarray(board.freqs, float),
            "Z_loop": np.array([[s.Z_loop for s in row] for row in sols]),
            "m": np.array([[s.m for s in row] for row in sols]),
            "iterations": np.array([[s.iterations for s in row] for row in sols]),
            "residual": np.array([[s.residual for s in row] for row in sols])}
