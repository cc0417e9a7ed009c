"""Interactive what-if edits on a solved board (GroundTruth: the fix search's candidate solves, suggest.py:318-325
and 452-465, on PlaneStack.with_branches, peec.py:1871-1923).

The base board is solved once per net and frequency.  An edit adds k branches (stitching vias, a decoupling
part; a part moved elsewhere is its removal, a parallel branch of the opposite impedance, plus its addition)
without joining separate pieces of copper.  Two ways to answer it:

* "bordered" (default): the edited system is the base system bordered by the k new branch currents,
      [K  F] [x]   [b    ]      F = the new branches' injections into the KCL rows,
      [G  Z] [i] = [b_new],     G x = -(V_a - V_b) across each new branch, Z = diag(z_new),
  so x = x_base - X_F i with X_F = K^-1 F (k solves of the base system per frequency, shared by every net)
  and i = (Z - G X_F)^-1 (b_new - G x_base), a k x k system per column.  Every device solve is a base solve
  with the base's own preconditioner; an edit costs k columns per frequency instead of one per net and
  frequency.  The edited residual is r' = r_base - r_F i on the base rows and zero on the new ones, so
  ||r'|| <= ||r_base|| + sum |i_j| ||r_F,j||, a bound known on the host; the base is solved to half the
  tolerance and X_F to border_tol (0.1) times it, and a column whose bound still misses the tolerance is solved on
  the derived stack from the composed solution.
* "derived": the derived stack (the base's factorisations plus a low-rank update of the Schur complement)
  solves every column, warm-started from the base's solution (the reference's way).  Its inner iterations
  run in FP32: an edit that shorts a weakly coupled piece of copper (a via from a plane island to ground at
  low frequency) removes, through the update, a potential mode that the base's FP32 sweeps carry at up to
  10^6 times the size of what remains, and a solve whose Krylov space starts from the warm start's residual
  (concentrated on the new branches) can stagnate in FP32 rounding.  Warm-started columns therefore run under
  an iteration budget (a multiple of the base solve's count) and are solved again from zero when they miss it.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import Callable

import numpy as np

from . import greens, stack as gs


@dataclass
class EditColumn:
    """One (net, frequency) answer of an edit: the loop impedance, moment and FP64 residual (for the bordered
    way a rigorous upper bound), and the full solution on demand (``solution()``: currents, potentials)."""
    f: float
    Z_loop: complex
    m: np.ndarray
    residual: float
    iterations: int
    make: Callable = field(repr=False, default=None)

    @property
    def L_loop(self) -> float:
        return self.Z_loop.imag / (2 * math.pi * self.f)

    def solution(self) -> gs.Solution:
        return self.make()


def _column(sol: gs.Solution) -> EditColumn:
    return EditColumn(sol.f, sol.Z_loop, sol.m, sol.residual, sol.iterations, lambda: sol)


def _real_times(A: np.ndarray, X: np.ndarray) -> np.ndarray:
    """A (m, n) real times each row of X (k, n) complex, as (m, k), without casting A to complex: the rows'
    real and imaginary parts are read in place (X's last axis contiguous)."""
    Xv = X.view(np.float64).reshape(X.shape[0], X.shape[1], 2)
    P = A @ Xv                                                       # (k, m, 2)
    return (P[..., 0] + 1j * P[..., 1]).T


@dataclass
class BorderPlan:
    """A bordered edit's border columns (frequencies, KCL injection vectors) and the step that composes its
    answers from their solve_batch results."""
    freqs: list
    Js: list
    compose: Callable


@dataclass
class EditResult:
    solutions: dict                     # (net, frequency) -> EditColumn
    seconds: float                      # wall time of the edit, derived stack to the last answer on the host
    iterations: list = field(default_factory=list)
    parts: dict = field(default_factory=dict)


class WhatIf:
    """A solved base board that answers edits.  routes: the base stack's RouteExcitations (nets); freqs: the
    frequencies the base is solved at (edits pick from them, so the base's factorisations serve every edit)."""

    def __init__(self, stack: gs.PlaneStack, routes: list, freqs, tol: float = 1e-5, max_cols: int = 32,
                 method: str = "bordered", warm_budget: float = 2.0, border_tol: float = 0.1, **solve_kw):
        if method not in ("bordered", "derived"):
            raise ValueError("method must be 'bordered' or 'derived'")
        self.stack = stack
        self.routes = list(routes)
        self.freqs = [float(f) for f in freqs]
        self.tol = tol
        self.max_cols = max_cols
        self.method = method
        self.border_tol = border_tol
        self.warm_budget = warm_budget
        self.kw = solve_kw
        self.base: dict = {}

    def _raw(self, stack, freqs: list, rhs_tops: list, Js: list, tol: float) -> list:
        """solve_batch in batches of max_cols: [(Ib, V, its, x, residual)]."""
        out = []
        for c0 in range(0, len(freqs), self.max_cols):
            sl = slice(c0, c0 + self.max_cols)
            out += stack.solve_batch(freqs[sl], rhs_tops[sl], Js[sl], tol=tol, **self.kw)
        return out

    def _solve(self, stack, routes: dict, cols: list, guesses=None, budget=None, tol=None) -> tuple:
        """Columns [(net, f)] on `stack` in batches of max_cols; returns (their Solutions in order, the
        indices of the warm-started columns that missed their budget and were solved again from zero, the
        solution vectors in the reference's unknown order)."""
        out, redo, xs = [], [], []
        tol = self.tol if tol is None else tol
        for c0 in range(0, len(cols), self.max_cols):
            part = cols[c0: c0 + self.max_cols]
            kw = dict(self.kw)
            failed = None
            if guesses is not None and budget is not None:
                kw["max_its"] = int(max(budget[c] for c in part))
                failed = []
            g = None if guesses is None else [guesses[c0 + q] for q in range(len(part))]
            res = stack.solve_batch([f for _, f in part], [routes[k].rhs_top(f) for k, f in part],
                                    [routes[k].J() for k, _ in part], tol=tol, guesses=g, failed=failed, **kw)
            if failed:
                again = stack.solve_batch([part[q][1] for q in failed], [routes[part[q][0]].rhs_top(part[q][1])
                                                                         for q in failed],
                                          [routes[part[q][0]].J() for q in failed], tol=tol, **self.kw)
                for q, r in zip(failed, again):
                    res[q] = (r[0], r[1], r[2] + res[q][2], r[3], r[4])
                redo += [c0 + q for q in failed]
            out += [routes[k].solution(f, Ib, V, its, r) for (k, f), (Ib, V, its, x, r) in zip(part, res)]
            xs += [r[3] for r in res]
        return out, redo, xs

    def baseline(self) -> float:
        """Solve every net at every frequency on the base stack; returns the seconds it took."""
        t0 = time.perf_counter()
        st = self.stack
        st.factorise(self.freqs, together=True)
        cols = [(k, f) for k in range(len(self.routes)) for f in self.freqs]
        tol = self.tol * (0.5 if self.method == "bordered" else 1.0)
        sols, _, xs = self._solve(st, dict(enumerate(self.routes)), cols, tol=tol)
        self.base = dict(zip(cols, sols))
        self.base_x = dict(zip(cols, xs))
        self.base_bnorm = {(k, f): float(np.linalg.norm(st.rhs_vector(self.routes[k].rhs_top(f), self.routes[k].J())))
                           for k, f in cols}
        self.base_psi_ib = {(k, f): complex(np.dot(self.routes[k].psi, x[: st.nb])) for (k, f), x in zip(cols, xs)}
        self.base_r_trace = {(k, f): float(greens.trace_resistance(self.routes[k].segments, f, st.sigma,
                                                                   self.routes[k].trace_t)) for k, f in cols}
        st.trim()                     # the baseline's workspace (all its columns) is not kept for the edits
        return time.perf_counter() - t0

    def evaluate(self, branches: list, nets, freqs, remove=()) -> EditResult:
        """The base plus `branches` and without the base's branches numbered in `remove` (a moved part: removed
        and added elsewhere), answered for the given nets (indices) at the given frequencies (a subset of the
        base's).  A removed branch is cancelled by a parallel one of the opposite impedance and the same coupling
        to the signal path: the pair's net current is zero, so the edited system's solution is the one without
        the branch (its unknowns keep the pair)."""
        if not self.base:
            raise RuntimeError("solve the baseline first")
        st = self.stack
        branches = list(branches) + [
            gs.Branch(st.branches[q].a, st.branches[q].b, (lambda f, z=st.branches[q].z: -z(f)),
                      f"-{st.branches[q].name}", st.branches[q].kind, st.branches[q].radius) for q in remove]
        keep = [b for b in branches if st.node_id(b.a) >= 0 and st.node_id(b.b) >= 0 and tuple(b.a) != tuple(b.b)]
        joins = any(st.full_label[st.node_id(b.a)] != st.full_label[st.node_id(b.b)] for b in keep)
        if self.method == "bordered" and keep and not joins:
            return self._bordered(keep, nets, freqs)
        return self._derived(branches, nets, freqs)

    def _bordered(self, extra: list, nets, freqs) -> EditResult:
        t0 = time.perf_counter()
        plan = self.border_plan(extra, nets, freqs)
        t1 = time.perf_counter()
        raw = self._raw(self.stack, plan.freqs, [np.zeros(self.stack.nb, complex)] * len(plan.Js), plan.Js,
                        self.tol * self.border_tol)
        t2 = time.perf_counter()
        res = plan.compose(raw)
        res.seconds = time.perf_counter() - t0
        res.parts.update({"derive_stack_s": t1 - t0, "border_solve_s": t2 - t1})
        return res

    def border_plan(self, extra: list, nets, freqs) -> "BorderPlan":
        """The device work of a bordered edit, apart from running it: its border columns (the base system's
        response to each new branch's unit injection at each frequency: frequencies and KCL vectors, solved to
        tol x border_tol), and the host step that composes the edit's answers from their solutions (a list of
        solve_batch results in the same order).  A server merges many edits' border columns into one device
        solve (serve.Server)."""
        st = self.stack
        dst = st.with_branches(extra, device=False)
        droutes = {k: self.routes[k].on(dst) for k in nets}
        nb, k, n_nodes = st.nb, len(extra), st.n_nodes
        kept = np.full(n_nodes, -1, np.int64)
        kept[np.flatnonzero(st.keep)] = np.arange(int(st.keep.sum()))
        na = np.array([st.node_id(b.a) for b in extra])
        nbn = np.array([st.node_id(b.b) for b in extra])
        ka, kb = kept[na], kept[nbn]
        arm = np.array([0.5 * np.cross(st.pos(b.a), st.pos(b.b)) for b in extra])        # (k, 3)
        freqs = [float(f) for f in freqs]
        # X_F: the base system's response to each new branch's unit injection (+1 at a, -1 at b), per frequency
        fcols = [(f, j) for f in freqs for j in range(k)]
        Js = []
        for f, j in fcols:
            J = np.zeros(n_nodes)
            J[na[j]] += 1.0
            J[nbn[j]] -= 1.0
            Js.append(J)
        return BorderPlan([f for f, _ in fcols], Js,
                          lambda raw: self._compose(extra, nets, freqs, dst, droutes, na, nbn, ka, kb, kept, arm,
                                                    fcols, raw))

    def _compose(self, extra, nets, freqs, dst, droutes, na, nbn, ka, kb, kept, arm, fcols, raw) -> EditResult:
        """A bordered edit's answers from its border solutions (raw: solve_batch results of its border
        columns)."""
        t2 = time.perf_counter()
        st = self.stack
        nb, k, n_nodes = st.nb, len(extra), st.n_nodes
        XF = {c: r[3] for c, r in zip(fcols, raw)}
        rF = {c: r[4] * np.sqrt(2.0) for c, r in zip(fcols, raw)}      # ||F_j|| = sqrt 2

        def at(v, idx):                        # rows of v at kept indices idx, zero where a node is not kept
            return np.where((idx >= 0).reshape((-1,) + (1,) * (v.ndim - 1)), v[np.maximum(idx, 0)], 0.0)

        # the real maps applied to the border solutions: the base's moment weights and the nets' couplings
        A = np.concatenate([st.moment_weights(), np.stack([self.routes[net].psi for net in nets])])
        cols_out, redo_cols, redo_x0 = {}, [], []
        for f in freqs:
            w = 2 * math.pi * f
            X = np.stack([XF[(f, j)] for j in range(k)])                  # (k, nb + n_keep), rows contiguous
            XI, VF = X[:, :nb], X[:, nb:]
            Sigma = np.diag([complex(b.z(f)) for b in extra]) + at(VF.T, ka) - at(VF.T, kb)
            rFf = np.array([rF[(f, j)] for j in range(k)])
            AX = _real_times(A, XI)
            MX, PX = AX[:3], AX[3:]                                       # (3, k) moments, (nets, k) psi . I
            for q, net in enumerate(nets):
                c = (net, f)
                base, xb = self.base[c], self.base_x[c]
                r = droutes[net]
                psi_new = r.psi[nb: nb + k]
                b_new = -1j * w * psi_new
                Vb = xb[nb:]
                i_new = np.linalg.solve(Sigma, b_new + at(Vb, ka) - at(Vb, kb))
                psi_ib = self.base_psi_ib[c] - PX[q] @ i_new + psi_new @ i_new
                v_inj = sum(a * (at(Vb, kept[[n]])[0] - at(VF.T, kept[[n]])[0] @ i_new) for n, a in r.injections)
                Z = complex(self.base_r_trace[c] + v_inj
                            + 1j * w * (r.L_trace + psi_ib))
                m = base.m - MX @ i_new + arm.T @ i_new
                bb = self.base_bnorm[c]
                bound = (base.residual * bb + float(np.abs(i_new) @ rFf)) / math.sqrt(bb * bb + float(np.vdot(b_new, b_new).real))

                def make(f=f, r=r, xb=xb, XI=XI, VF=VF, i_new=i_new, bound=bound):
                    V = np.zeros(n_nodes, complex)
                    V[st.keep] = xb[nb:] - i_new @ VF
                    return r.solution(f, np.concatenate([xb[:nb] - i_new @ XI, i_new]), V, 0, bound)
                cols_out[c] = EditColumn(f, Z, m, bound, 0, make)
                if not bound <= self.tol:
                    redo_cols.append(c)
                    redo_x0.append(np.concatenate([xb[:nb] - i_new @ XI, i_new, Vb - i_new @ VF]))
        t3 = time.perf_counter()
        if redo_cols:
            # columns whose bound misses the tolerance: the derived stack, from the composed solution
            ddst = st.with_branches(extra)
            drr = {net: self.routes[net].on(ddst) for net in nets}
            out, _, _ = self._solve(ddst, drr, redo_cols, [[x] for x in redo_x0],
                                    {c: self.warm_budget * self.base[c].iterations + self.kw.get("restart", 50)
                                     for c in redo_cols})
            cols_out.update((c, _column(sol)) for c, sol in zip(redo_cols, out))
        t4 = time.perf_counter()
        cols = [(net, f) for net in nets for f in freqs]
        return EditResult({c: cols_out[c] for c in cols}, t4 - t2, [r[2] for r in raw],
                          {"compose_s": t3 - t2, "redo_s": t4 - t3, "border_columns": len(fcols),
                           "cold_redo": len(redo_cols)})

    def _derived(self, branches: list, nets, freqs) -> EditResult:
        t0 = time.perf_counter()
        dst = self.stack.with_branches(branches)
        droutes = {k: self.routes[k].on(dst) for k in nets}
        t1 = time.perf_counter()
        cols = [(k, float(f)) for k in nets for f in freqs]
        guesses = [[dst.map_state(self.base_x[c], self.stack)] for c in cols]
        dst.factorise([f for _, f in cols], together=True)
        t2 = time.perf_counter()
        budget = {c: self.warm_budget * self.base[c].iterations + self.kw.get("restart", 50) for c in cols}
        sols, redo, _ = self._solve(dst, droutes, cols, guesses, budget)
        dst.release_operators()           # its device memory now, not when the collector finds the stack
        dst.trim()
        t3 = time.perf_counter()
        return EditResult({c: _column(sol) for c, sol in zip(cols, sols)}, t3 - t0, [s.iterations for s in sols],
                          {"derive_stack_s": t1 - t0, "operators_s": t2 - t1, "solve_s": t3 - t2,
                           "cold_redo": len(redo)})
