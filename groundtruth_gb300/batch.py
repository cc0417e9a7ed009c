"""Many boards solved together on one GPU: the uneven-batch workload's driver (boards of different raster sizes,
sheet counts, nets and frequencies, each with its own factorisations; GroundTruth runs such boards as separate
simulate jobs under its task scheduler and memory admission, analysis/simulate.py:3930-4030).

Boards are grouped by their padded FFT sizes and sheet counts (the L_p kernels' compile-time shapes) and taken
largest first.  Up to `concurrency` boards are in flight at once, each on a host thread of its own with a CUDA
stream of its own: a board factorises its frequencies, scatters its right-hand sides into device memory and
runs one batched device solve of all its columns (gt_solve_device), so the kernels of small boards, which alone
fill only a few SMs, overlap on the device.  A board is admitted when its device memory (its factorisations,
kept as FP32 panels only, and the workspace and dense vectors of all its columns) fits the budget left by the
boards in flight; a board larger than the whole budget runs alone within it, factorising its frequencies in
chunks and solving their columns in batches that fit.  A board's result does not depend on what else
is in flight: its kernels see only its own buffers and run in the same order on its stream.
"""
from __future__ import annotations

import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import native
from . import stack as gs


@dataclass
class BoardJob:
    """One board's stack, excitations and columns (net index, frequency index)."""
    name: str
    stack: gs.PlaneStack
    routes: list
    freqs: list
    tol: float
    cols: list = field(default_factory=list)

    @property
    def group(self) -> tuple:
        st = self.stack
        return (tuple(st.P["x"]), tuple(st.P["y"]), st.n_sheets)


@dataclass
class BoardResult:
    name: str
    x: np.ndarray                # (ncol, n_compact) solutions in the reference's order
    its: np.ndarray
    residual: np.ndarray
    Z: np.ndarray                # per column Z_loop
    seconds: float               # wall time of the board's factorisation + solve on its stream
    factorise_s: float


def prepare(boards: list) -> list:
    """BoardJobs of synth.Boards (host setup: topology, symbolic analysis, spectra; not part of a solve)."""
    jobs = []
    for b in boards:
        st, routes = gs.from_board(b)
        freqs = [float(f) for f in b.freqs]
        jobs.append(BoardJob(b.name, st, routes, freqs, float(b.tol),
                             [(k, q) for k in range(len(routes)) for q in range(len(freqs))]))
    return jobs


class MemoryBudget:
    """Device bytes handed out to the boards in flight (a counting lock over a byte budget)."""

    def __init__(self, budget: int):
        self.budget = int(budget)
        self.used = 0
        self.cv = threading.Condition()

    def acquire(self, n: int) -> int:
        n = min(int(n), self.budget)             # a board larger than the budget runs alone
        with self.cv:
            while self.used + n > self.budget:
                self.cv.wait()
            self.used += n
        return n

    def release(self, n: int):
        with self.cv:
            self.used -= n
            self.cv.notify_all()


def _column_bytes(job: BoardJob, restart: int, precision: str) -> int:
    """Device bytes one more column adds to a solve: its workspace share and its dense right-hand side and
    solution."""
    h = job.stack.handle
    one = native.memory(h, 1, restart, precision)["need"]
    return int(native.memory(h, 2, restart, precision)["need"] - one + 2 * h.n_dense * 16)


def _device_bytes(job: BoardJob, restart: int, precision: str) -> int:
    """What a board asks of the budget: its factorisations and all its columns at once."""
    return int(job.stack.factorisation_bytes(len(job.freqs)) + len(job.cols) * _column_bytes(job, restart, precision))


def solve_board(job: BoardJob, stream=None, restart: int = 50, precision: str = "mixed", max_its: int = 4000,
                avail_bytes: Optional[int] = None) -> BoardResult:
    """Factorise a board's frequencies and solve all its columns on `stream` (a torch.cuda.Stream; the current
    one when None) within avail_bytes of device memory (default: 90 % of the free memory): the factorisations
    keep their FP32 panels only and are made in chunks of frequencies that take at most half the memory, each
    chunk's columns solved in batches that fit the rest, the chunk's factorisations released after it."""
    import torch
    st = job.stack
    st.fp32_panels = True
    stream = stream or torch.cuda.current_stream()
    n = st.handle.n_dense
    ncol = len(job.cols)
    x = np.zeros((ncol, st.handle.n_compact), complex)
    its = np.zeros(ncol, np.int32)
    res = np.zeros(ncol)
    t_fact = 0.0
    with torch.cuda.stream(stream):
        t0 = time.perf_counter()
        avail = int(avail_bytes if avail_bytes is not None else 0.9 * native.memory(st.handle, 1)["free"])
        nq = len(job.freqs)
        chunk = max(1, min(nq, int(0.5 * avail // max(st.factorisation_bytes(1), 1))))
        per_col = _column_bytes(job, restart, precision)
        for q0 in range(0, nq, chunk):
            qs = list(range(q0, min(nq, q0 + chunk)))
            tf = time.perf_counter()
            ops = st.factorise([job.freqs[q] for q in qs], together=True)
            t_fact += time.perf_counter() - tf
            obj = ops[0][0]
            prec = "mixed_pc64" if precision == "mixed" and getattr(obj, "stiff", False) else precision
            mine = [c for c, (_, q) in enumerate(job.cols) if q0 <= q < q0 + len(qs)]
            room = max(avail - st.resident_bytes(len(qs)), per_col)
            step = max(1, min(len(mine), int(room // per_col), st.columns_that_fit(len(mine), restart, prec)))
            for c0 in range(0, len(mine), step):
                sel = mine[c0: c0 + step]
                m = len(sel)
                rhs = np.stack([st.rhs_vector(job.routes[k].rhs_top(job.freqs[q]), job.routes[k].J())
                                for k, q in (job.cols[c] for c in sel)])
                col_op = np.array([ops[job.cols[c][1] - q0][1] for c in sel], np.int32)
                B = torch.zeros((m, n), dtype=torch.complex128, device="cuda")
                X = torch.zeros_like(B)
                st.handle.to_dense(rhs, B.data_ptr(), stream.cuda_stream)
                its[sel], res[sel] = st.handle.solve_device(obj, col_op, B.data_ptr(), X.data_ptr(), job.tol,
                                                            restart=restart, max_its=max_its, precision=prec,
                                                            stream=stream.cuda_stream, reorth=0.0)
                x[sel] = st.handle.to_compact(X.data_ptr(), m, stream.cuda_stream)
                del B, X
            stream.synchronize()
            del ops, obj
            st.release_operators()
        st.trim()                     # the board's workspace goes back before the next board takes memory
        seconds = time.perf_counter() - t0
    Z = np.zeros(ncol, complex)
    for c, (k, q) in enumerate(job.cols):
        V = np.zeros(st.n_nodes, complex)
        V[st.keep] = x[c, st.nb:]
        Z[c] = job.routes[k].solution(job.freqs[q], x[c, : st.nb], V, int(its[c])).Z_loop
    return BoardResult(job.name, x, its, res, Z, seconds, t_fact)


def solve_all(jobs: list, concurrency: int = 8, budget_bytes: Optional[int] = None, restart: int = 50,
              precision: str = "mixed") -> list:
    """Solve every board, up to `concurrency` at once on streams of their own, admitted against budget_bytes of
    device memory (default: 90 % of the free memory).  Returns the BoardResults in the jobs' order."""
    import torch
    if budget_bytes is None:
        budget_bytes = int(0.9 * native.memory(jobs[0].stack.handle, 1)["free"])
    budget = MemoryBudget(budget_bytes)
    order = sorted(range(len(jobs)), key=lambda i: (jobs[i].group, jobs[i].stack.handle.n_dense), reverse=True)
    local = threading.local()

    def run(i):
        job = jobs[i]
        if not hasattr(local, "stream"):
            local.stream = torch.cuda.Stream()
        need = budget.acquire(_device_bytes(job, restart, precision))
        try:
            return i, solve_board(job, local.stream, restart, precision, avail_bytes=need)
        finally:
            budget.release(need)

    out = [None] * len(jobs)
    if concurrency <= 1:
        for i in order:
            out[i] = run(i)[1]
        return out
    with ThreadPoolExecutor(concurrency) as ex:
        for i, r in ex.map(run, order):
            out[i] = r
    return out
