"""Interactive what-if edits on a solved board (GroundTruth: the fix search's candidate solves, suggest.py:318-325
and 452-465, on PlaneStack.with_branches, peec.py:1871-1923).

The base board is solved once per net and frequency.  Each edit (added stitching vias, an added decoupling part)
becomes a derived stack that reuses the base's factorisations through a low-rank (Woodbury) update, and its
solves start from the base's solutions mapped onto the derived stack's unknowns (the new branches at zero
current), all columns of an edit in as few device batches as the device memory budget allows.

The inner iterations run in FP32.  An edit that shorts a weakly coupled piece of copper (a via from a plane
island to ground at low frequency) removes, through the low-rank update, a potential mode that the base's
FP32 solve carries at up to 10^6 times the size of what remains; the remainder then drowns in FP32 rounding
when the Krylov space starts from the warm start's residual (concentrated on the new branches), and such a
solve stagnates.  Warm-started columns therefore run under an iteration budget (a multiple of the base
solve's count), and the columns that miss it are solved again from zero, which converges like a fresh
factorisation of the edited board."""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import stack as gs


@dataclass
class EditResult:
    solutions: dict                     # (net, frequency) -> stack.Solution
    seconds: float                      # wall time of the edit, derived stack to the last solution on the host
    iterations: list = field(default_factory=list)
    parts: dict = field(default_factory=dict)


class WhatIf:
    """A solved base board that answers edits.  routes: the base stack's RouteExcitations (nets); freqs: the
    frequencies the base is solved at (edits pick from them, so the base's factorisations serve every edit)."""

    def __init__(self, stack: gs.PlaneStack, routes: list, freqs, tol: float = 1e-5, max_cols: int = 32,
                 warm_budget: float = 2.0, **solve_kw):
        self.stack = stack
        self.routes = list(routes)
        self.freqs = [float(f) for f in freqs]
        self.tol = tol
        self.max_cols = max_cols
        self.warm_budget = warm_budget
        self.kw = solve_kw
        self.base: dict = {}

    def _solve(self, stack, routes: dict, cols: list, guesses=None, budget=None) -> tuple:
        """Columns [(net, f)] on `stack` in batches of max_cols; returns (their Solutions in order, the
        indices of the warm-started columns that missed their budget and were solved again from zero)."""
        out, redo = [], []
        for c0 in range(0, len(cols), self.max_cols):
            part = cols[c0: c0 + self.max_cols]
            kw = dict(self.kw)
            failed = None
            if guesses is not None and budget is not None:
                kw["max_its"] = int(max(budget[c] for c in part))
                failed = []
            g = None if guesses is None else [guesses[c0 + q] for q in range(len(part))]
            res = stack.solve_batch([f for _, f in part], [routes[k].rhs_top(f) for k, f in part],
                                    [routes[k].J() for k, _ in part], tol=self.tol, guesses=g, failed=failed, **kw)
            if failed:
                again = stack.solve_batch([part[q][1] for q in failed], [routes[part[q][0]].rhs_top(part[q][1])
                                                                         for q in failed],
                                          [routes[part[q][0]].J() for q in failed], tol=self.tol, **self.kw)
                for q, r in zip(failed, again):
                    res[q] = (r[0], r[1], r[2] + res[q][2], r[3], r[4])
                redo += [c0 + q for q in failed]
            out += [routes[k].solution(f, Ib, V, its, r) for (k, f), (Ib, V, its, x, r) in zip(part, res)]
        return out, redo

    def baseline(self) -> float:
        """Solve every net at every frequency on the base stack; returns the seconds it took."""
        t0 = time.perf_counter()
        self.stack.factorise(self.freqs, together=True)
        cols = [(k, f) for k in range(len(self.routes)) for f in self.freqs]
        sols, _ = self._solve(self.stack, dict(enumerate(self.routes)), cols)
        self.base = dict(zip(cols, sols))
        return time.perf_counter() - t0

    def evaluate(self, branches: list, nets, freqs) -> EditResult:
        """The base plus `branches`, solved for the given nets (indices) at the given frequencies (a subset of
        the base's), warm-started from the base's solutions."""
        if not self.base:
            raise RuntimeError("solve the baseline first")
        t0 = time.perf_counter()
        dst = self.stack.with_branches(branches)
        droutes = {k: self.routes[k].on(dst) for k in nets}
        t1 = time.perf_counter()
        cols = [(k, float(f)) for k in nets for f in freqs]
        guesses = [[dst.map_state(self.base[c].state_for(self.stack), self.stack)] for c in cols]
        dst.factorise([f for _, f in cols], together=True)
        t2 = time.perf_counter()
        budget = {c: self.warm_budget * self.base[c].iterations + self.kw.get("restart", 50) for c in cols}
        sols, redo = self._solve(dst, droutes, cols, guesses, budget)
        t3 = time.perf_counter()
        return EditResult(dict(zip(cols, sols)), t3 - t0, [s.iterations for s in sols],
                          {"derive_stack_s": t1 - t0, "operators_s": t2 - t1, "solve_s": t3 - t2,
                           "cold_redo": len(redo)})
