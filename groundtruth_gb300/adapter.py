"""GroundTruth's own solver with the GB300 solve dropped in (the seam of PlaneStack.solve, peec.py:2513-2558).

install(peec) replaces ``peec.PlaneStack.solve`` by one that builds, once per stack, this package's device stack
from the same layers (their grids), branches, plane pairs, conductivity, preconditioner and screening flag, and
solves there: ``RouteExcitation.solve``, the simulation's ``solve_at`` and the fix search's calls run unchanged
and get ``(Ib, V, its, x)`` in the reference's unknown order.  A guess (warm start) is passed through; a solve
that misses its tolerance raises the reference's own ``SolverError``.  uninstall(peec) puts the original back.

The device stack keeps the reference stack's factorisations on the GPU between solves (its operator cache); a
derived stack of the reference (``with_branches``) gets a device stack of its own."""
from __future__ import annotations

from . import stack as gs

_ATTR = "_gb300_stack"


def _device_stack(st) -> gs.PlaneStack:
    dev = st.__dict__.get(_ATTR)
    if dev is None:
        dev = gs.PlaneStack(list(st.layers), list(st.branches), list(st.pairs), st.sigma, precond=st.precond_mode,
                            screen=st.screen)
        st.__dict__[_ATTR] = dev
    return dev


def install(peec) -> None:
    """Route ``peec.PlaneStack.solve`` through the GB300 solve (idempotent)."""
    cls = peec.PlaneStack
    if getattr(cls, "_gb300_original_solve", None) is not None:
        return

    def solve(self, f, rhs_top, J, tol=1e-5, max_cycles=8, guess=None):
        """PlaneStack.solve (peec.py:2513) on the GPU: (Ib (nb), V (n_nodes), its, x)."""
        try:
            Ib, V, its, x, _ = _device_stack(self).solve_batch([f], [rhs_top], [J], tol=tol, max_cycles=max_cycles,
                                                               guesses=[guess])[0]
        except gs.SolverError as e:
            raise peec.SolverError(str(e)) from e
        return Ib, V, its, x

    cls._gb300_original_solve = cls.solve
    cls.solve = solve


def uninstall(peec) -> None:
    """Put the reference's own ``PlaneStack.solve`` back."""
    cls = peec.PlaneStack
    original = getattr(cls, "_gb300_original_solve", None)
    if original is not None:
        cls.solve = original
        cls._gb300_original_solve = None
