"""The drop-in seam on GroundTruth's own solver (peec.py:2513-2558): adapter.install routes the reference's
PlaneStack.solve through this package's stack, and the reference's RouteExcitation.solve returns what the
reference's own solve returns.  The reference is imported from its source tree (shapely stubbed: the boards are
given as grids), so this runs only where the source is; the device solve is stood in for by the oracle, on the
CPU: what is checked is the seam (arguments, unknown order, outputs, errors)."""
import os
import sys
import types
from pathlib import Path

import numpy as np
import pytest

from groundtruth_gb300 import adapter, stack as gs, synth
from oracle import peec_oracle as po

REFERENCE = Path(os.environ.get("GT_REFERENCE_SRC", "/root/reference")) / "src"


@pytest.fixture
def peec(monkeypatch):
    if not (REFERENCE / "groundtruth" / "solver" / "peec.py").exists():
        pytest.skip("the reference's source is not here")
    sys.modules.setdefault("shapely", types.ModuleType("shapely"))
    monkeypatch.syspath_prepend(str(REFERENCE))
    from groundtruth.solver import peec as module
    yield module
    adapter.uninstall(module)


def _oracle_backed(monkeypatch):
    """This package's stacks on the host, their solves by the oracle (FP64, the reference's algorithm)."""
    init = gs.PlaneStack.__init__

    def host(self, *a, _device=True, **k):
        init(self, *a, _device=False, **k)

    def solve_batch(self, freqs, rhs_tops, Js, tol=1e-5, guesses=None, failed=None, **kw):
        ost = self.__dict__.get("_oracle")
        if ost is None:
            wk = ("wx", "wy", "ox", "oy", "rx", "ry")
            layers = [po.OLayer(l.z, l.thickness, l.grid.node, l.grid.xb, l.grid.yb,
                                {k: getattr(l.grid, k) for k in wk if getattr(l.grid, k, None) is not None} or None,
                                getattr(l.grid, "fill", None)) for l in self.layers]
            ost = self.__dict__["_oracle"] = po.OracleStack(layers, self.d, self.branches_all, self.pairs, self.sigma,
                                                            self.precond_mode, self.screen)
        out = []
        for f, top, J in zip(freqs, rhs_tops, Js):
            Ib, V, its, x = ost.solve(f, np.asarray(top, complex), np.asarray(J, float), tol=tol)
            out.append((Ib, V, its, x, 0.0))
        return out
    monkeypatch.setattr(gs.PlaneStack, "__init__", host)
    monkeypatch.setattr(gs.PlaneStack, "solve_batch", solve_batch)


def _reference_board(peec, board):
    grids = [peec.Grid(0.0, 0.0, board.d * 1e3, board.nx, board.ny, l.node.copy(), l.xb.copy(), l.yb.copy(),
                       **{k: np.array(v, float) for k, v in (l.widths or {}).items()}) for l in board.layers]
    layers = [peec.PlaneLayer(l.name, l.z, g, l.thickness) for l, g in zip(board.layers, grids)]
    branches = [peec.Branch(b.a, b.b, (lambda f, b=b: b.z(f)), f"br{n}", b.kind, b.radius)
                for n, b in enumerate(board.branches)]
    pairs = [peec.PlanePair(p.upper, p.lower, p.c_per_area, p.tan_delta) for p in board.pairs]
    st = peec.PlaneStack(layers, branches, pairs, board.sigma, precond=board.precond, screen=board.screen)
    routes = [peec.RouteExcitation(st, [peec.TraceSegment(s[0:3].copy(), s[3:6].copy(), float(s[6]), float(s[7]))
                                        for s in net.segments], net.driver, net.receiver, net.trace_t)
              for net in board.nets]
    return st, routes


@pytest.mark.parametrize("name", ["small_pair", "necked_faces"])
def test_the_reference_solves_through_the_seam(peec, monkeypatch, name):
    board = getattr(synth, name)()
    f = float(board.freqs[1])
    st, routes = _reference_board(peec, board)
    own = routes[0].solve(f)                               # the reference's own solve (tol 1e-5)
    _oracle_backed(monkeypatch)
    adapter.install(peec)
    st2, routes2 = _reference_board(peec, board)
    got = routes2[0].solve(f)
    assert isinstance(st2.__dict__.get("_gb300_stack"), gs.PlaneStack)
    assert abs(got.Z_loop - own.Z_loop) <= 1e-4 * abs(own.Z_loop)
    assert np.linalg.norm(got.I_x - own.I_x) <= 1e-3 * np.linalg.norm(own.I_x)
    again = routes2[0].solve(float(board.freqs[0]))        # the same device stack serves the next frequency
    assert st2.__dict__["_gb300_stack"] is not None and np.isfinite(again.Z_loop)
    adapter.uninstall(peec)
    assert routes2[0].solve(f).Z_loop == pytest.approx(own.Z_loop, rel=1e-12)


def test_a_solve_that_misses_raises_the_reference_s_error(peec, monkeypatch):
    board = synth.small_pair()
    _oracle_backed(monkeypatch)

    def missing(self, freqs, *a, **k):
        raise gs.SolverError(f"GMRES did not converge at {freqs[0]:.4g} Hz")
    monkeypatch.setattr(gs.PlaneStack, "solve_batch", missing)
    adapter.install(peec)
    st, routes = _reference_board(peec, board)
    with pytest.raises(peec.SolverError, match="did not converge"):
        routes[0].solve(float(board.freqs[0]))
