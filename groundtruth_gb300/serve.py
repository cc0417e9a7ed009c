"""A what-if request server with continuous batching on resident geometries (the serving workload; GroundTruth's
interactive candidate solves, suggest.py:318-325 and 452-465, on PlaneStack.with_branches, peec.py:1871-1923).

Each geometry stays resident on the device with its kernel spectra, its factorisations at the served
frequencies and its base solutions (whatif.WhatIf).  Requests arrive on any thread (submit) and return a Future.
One batcher thread takes every request waiting when the device is free, up to the columns the memory budget
admits (the budget governs the requests' working memory, the Krylov workspace and vectors per column; the
resident geometries are outside it and reported as resident_bytes), and runs them as ONE device solve per
geometry:

* an edit that adds stitching vias or moves a decoupling part (a removal plus an addition) contributes its
  border columns, the base system's response to each new branch's unit injection at each asked frequency, to
  the base geometry's batch; its answers are composed on the host from them (WhatIf.border_plan);
* a slot toggle is the base board with its slot filled or cut again, a geometry of its own (resident beside
  the base): its nets' columns join that geometry's batch.

The geometries' batches run side by side on CUDA streams of their own.  Requests that arrive while a batch is on
the device wait for the next one, which takes them together with everything else that arrived meanwhile, so a
burst is served in a few large batches instead of one request after another.  A request's answers do not depend
on what it was batched with: the device arithmetic of a column is its own.
"""
from __future__ import annotations

import queue
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import native
from .whatif import EditColumn, EditResult, WhatIf


@dataclass
class Request:
    """An edit: `branches` added (stitching vias, a decoupling part) and the base's branches numbered `remove`
    taken away (a moved part) on the base geometry, or, with `geometry` naming another resident geometry, no edit
    on that one (a slot toggle); answered for nets (indices) at freqs (a subset of the served frequencies)."""
    nets: list
    freqs: list
    branches: list = field(default_factory=list)
    remove: list = field(default_factory=list)
    geometry: str = "base"
    arrival: float = 0.0


@dataclass
class Answer:
    result: EditResult
    latency_s: float             # arrival to answer
    queued_s: float              # arrival to its batch's start
    batch_requests: int          # requests in its batch
    batch_columns: int           # device columns of its batch


class Server:
    """Serves Requests on resident geometries {name: WhatIf} (their baselines solved) with continuous batching,
    the requests' working memory admitted against budget_bytes."""

    def __init__(self, geometries: dict, budget_bytes: float = 120e9, max_cols: Optional[int] = None,
                 restart: int = 50):
        import torch
        if "base" not in geometries:
            raise ValueError("the geometries need a 'base'")
        self.geo = dict(geometries)
        self.restart = restart
        self.q: "queue.Queue" = queue.Queue()
        self.streams = {name: torch.cuda.Stream() for name in self.geo}
        # columns per batch: every geometry keeps a workspace as wide as the widest batch it took, so the budget
        # holds max_cols columns of each geometry's workspace
        one = per = 0
        for w in self.geo.values():
            w.stack.trim()                         # what the baselines left behind
            o = native.memory(w.stack.handle, 1, restart)["need"]
            one += o
            per += max(native.memory(w.stack.handle, 2, restart)["need"] - o, 1)
        fit = int((budget_bytes - one) // per) + 1
        self.max_cols = max(1, min(fit, max_cols or fit))
        for w in self.geo.values():          # every device solve of a geometry in batches of at most that
            w.max_cols = self.max_cols
        self.resident_bytes = sum(w.stack.resident_bytes(len(w.freqs)) for w in self.geo.values())
        self.batches = []
        self._stop = threading.Event()
        self._thread = threading.Thread(target=self._loop, name="what-if batcher", daemon=True)
        self._thread.start()

    # ------------------------------------------------------------------ client side
    def submit(self, req: Request) -> Future:
        req.arrival = req.arrival or time.perf_counter()
        fut: Future = Future()
        self.q.put((req, fut))
        return fut

    def close(self):
        self._stop.set()
        self.q.put(None)
        self._thread.join()

    # ------------------------------------------------------------------ batcher
    def _columns(self, req: Request) -> int:
        """Device columns of a request: its nets at its frequencies on another geometry or on a derived stack
        (an edit that joins separate copper), else its border columns."""
        if req.geometry != "base" or self._joins(self.geo["base"], req):
            return len(req.nets) * len(req.freqs)
        return (len(req.branches) + len(req.remove)) * len(req.freqs)

    @staticmethod
    def _joins(wi: WhatIf, req: Request) -> bool:
        """True when the edit needs the derived stack: a new branch off the base's nodes or between separate
        pieces of copper."""
        st = wi.stack
        if not req.branches and not req.remove:
            return True
        for b in req.branches:
            ia, ib = st.node_id(b.a), st.node_id(b.b)
            if ia < 0 or ib < 0 or tuple(b.a) == tuple(b.b) or st.full_label[ia] != st.full_label[ib]:
                return True
        return False

    def _loop(self):
        carry = []
        while not self._stop.is_set():
            items, carry = carry, []
            if not items:
                got = self.q.get()
                if got is None:
                    break
                items = [got]
            while True:                       # everything that is waiting now
                try:
                    got = self.q.get_nowait()
                except queue.Empty:
                    break
                if got is None:
                    self._stop.set()
                    break
                items.append(got)
            batch, cols = [], 0
            for it in items:                  # admitted in arrival order while the budget's columns last
                c = self._columns(it[0])
                if batch and cols + c > self.max_cols:
                    carry.append(it)
                else:
                    batch.append(it)
                    cols += c
            try:
                self._run(batch, cols)
            except Exception as e:            # the batch's requests fail, the server goes on
                for _, fut in batch:
                    if not fut.done():
                        fut.set_exception(e)
        for _, fut in carry:
            if not fut.done():
                fut.set_exception(RuntimeError("the server closed"))

    def _run(self, batch: list, ncols: int):
        import torch
        t0 = time.perf_counter()
        per_geo: dict = {}
        for req, fut in batch:
            per_geo.setdefault(req.geometry, []).append((req, fut))
        results = {}

        def run_geometry(name, items):
            wi = self.geo[name]
            st = wi.stack
            with torch.cuda.stream(self.streams[name]):
                if name == "base":
                    plans, freqs, Js, direct = [], [], [], []
                    for req, fut in items:
                        plan = self._plan(wi, req)
                        if plan is None:
                            direct.append((req, fut))
                            continue
                        plans.append((fut, plan, len(freqs)))
                        freqs += plan.freqs
                        Js += plan.Js
                    raw = wi._raw(st, freqs, [np.zeros(st.nb, complex)] * len(Js), Js, wi.tol * wi.border_tol) \
                        if Js else []
                    for fut, plan, c0 in plans:
                        results[id(fut)] = plan.compose(raw[c0: c0 + len(plan.Js)])
                    if direct:
                        st.trim()              # the derived stacks' workspaces take the base's place
                    for req, fut in direct:    # an edit that joins separate copper: the derived stack
                        results[id(fut)] = wi.evaluate(req.branches, req.nets, req.freqs, remove=req.remove)
                else:
                    cols = [(k, float(f)) for req, _ in items for k in req.nets for f in req.freqs]
                    sols, _, _ = wi._solve(st, dict(enumerate(wi.routes)), cols, tol=wi.tol)
                    at = 0
                    for req, fut in items:
                        keys = [(k, float(f)) for k in req.nets for f in req.freqs]
                        mine = sols[at: at + len(keys)]
                        at += len(keys)
                        out = {c: EditColumn(s.f, s.Z_loop, s.m, s.residual, s.iterations, lambda s=s: s)
                               for c, s in zip(keys, mine)}
                        results[id(fut)] = EditResult(out, 0.0, [s.iterations for s in mine], {})
                self.streams[name].synchronize()

        threads = [threading.Thread(target=self._guard, args=(run_geometry, name, items))
                   for name, items in per_geo.items()]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        t1 = time.perf_counter()
        self.batches.append({"start": t0, "seconds": t1 - t0, "requests": len(batch), "columns": ncols})
        for req, fut in batch:
            if fut.done():
                continue
            res = results.get(id(fut))
            if res is None:
                fut.set_exception(RuntimeError("the request's batch did not answer it"))
                continue
            res.seconds = t1 - req.arrival
            fut.set_result(Answer(res, t1 - req.arrival, t0 - req.arrival, len(batch), ncols))

    @staticmethod
    def _guard(fn, name, items):
        try:
            fn(name, items)
        except Exception as e:
            for _, fut in items:
                if not fut.done():
                    fut.set_exception(e)

    @staticmethod
    def _plan(wi: WhatIf, req: Request):
        """The request's border plan on the base, or None when it must go through the derived stack (an edit
        that joins separate pieces of copper, or a branch off the base's nodes)."""
        from . import stack as gs
        st = wi.stack
        extra = list(req.branches) + [
            gs.Branch(st.branches[q].a, st.branches[q].b, (lambda f, z=st.branches[q].z: -z(f)),
                      f"-{st.branches[q].name}", st.branches[q].kind, st.branches[q].radius) for q in req.remove]
        keep = [b for b in extra if st.node_id(b.a) >= 0 and st.node_id(b.b) >= 0 and tuple(b.a) != tuple(b.b)]
        if not keep or len(keep) != len(extra):
            return None
        if any(st.full_label[st.node_id(b.a)] != st.full_label[st.node_id(b.b)] for b in keep):
            return None
        return wi.border_plan(keep, req.nets, req.freqs)
