"""The reference's analytic known-answer cases for this solve (tests/test_solver.py:31-88 of GroundTruth),
restated on a 40 x 20 mm plane under a microstrip (synth.microstrip): the strip kernel's symmetry and self term,
the return current under the trace against image theory, the loop inductance against Wheeler's formula and
the moment against the loop's area, current spreading at low frequency, a slot's monotonic effect, a cut from
the edge turning the loop into the board plane, and a fully cut plane refused.  Each runs on the oracle (CPU)
and, marked gpu, through the CUDA library."""
import math

import numpy as np
import pytest

from groundtruth_gb300 import greens, stack as gs, synth
from oracle import peec_oracle as po
from test_oracle_golden import oracle_routes, oracle_stack

H, W = 0.5e-3, 0.2e-3


def _oracle(board, f):
    r = oracle_routes(oracle_stack(board), board)[0]
    out = r.solve(f, tol=board.tol)
    return out["I_x"], out["Z_loop"], out["m"]


def _device(board, f):
    st, routes = gs.from_board(board)
    sol = routes[0].solve(f, tol=board.tol)
    return sol.I_x, sol.Z_loop, sol.m


SOLVERS = [pytest.param(_oracle, id="oracle"), pytest.param(_device, id="gpu", marks=pytest.mark.gpu)]


def test_kernel_symmetry_and_self_term():
    """test_solver.py:31-37: the kernel is even, its centre the numeric self term, it falls off with distance
    and far away equals the filament formula."""
    for mod in (greens, po):
        K = mod.strip_kernel(6, 6, 1e-3, 0.0)
        assert np.allclose(K, K[::-1, ::-1])
        assert K[5, 5] == pytest.approx(float(mod.strip_self_numeric(1e-3, 1e-3)))
        assert K[5, 5] > K[6, 5] > K[7, 5] > 0
        assert K[5, 10] == pytest.approx(float(mod.filament_mutual(1e-3, 0.0, 5e-3)), rel=1e-3)


@pytest.mark.parametrize("solve", SOLVERS)
def test_return_current_follows_image_theory(solve):
    """test_solver.py:40-49: the plane current under the trace at x = 20 mm is H / (pi (H^2 + y^2)) within
    6 % for |y| <= 2 mm, and all of the current returns."""
    b = synth.microstrip()
    I_x, Z, m = solve(b, 1e8)
    i = 80
    y = np.arange(b.ny) * b.d - 10e-3
    K = -I_x[0, i, :].real / b.d
    analytic = H / (math.pi * (H * H + y * y))
    near = np.abs(y) <= 2e-3
    assert np.allclose(K[near], analytic[near], rtol=0.06)
    assert I_x[0, i, :].sum().real == pytest.approx(-1.0, abs=1e-3)


@pytest.mark.parametrize("solve", SOLVERS)
def test_loop_inductance_and_moment(solve):
    """test_solver.py:52-57: L_loop within 3 % of Wheeler's microstrip over 30 mm, |m| the loop's area."""
    b = synth.microstrip()
    I_x, Z, m = solve(b, 1e8)
    L = Z.imag / (2 * math.pi * 1e8)
    wheeler = 2e-7 * math.log(8 * H / W + W / (4 * H)) * 0.030
    assert L == pytest.approx(wheeler, rel=0.03)
    assert np.linalg.norm(m) == pytest.approx(30e-3 * H, rel=0.01)


@pytest.mark.parametrize("solve", SOLVERS)
def test_low_frequency_current_spreads(solve):
    """test_solver.py:60-66: at 1 kHz the return current spreads (resistive), less than a fifth of the 100 MHz
    current flows under the trace, and the loop inductance is higher."""
    b = synth.microstrip(f=(1e3, 1e8))
    lf, hf = solve(b, 1e3), solve(b, 1e8)
    assert abs(lf[0][0, 80, 40]) < 0.2 * abs(hf[0][0, 80, 40])
    assert lf[1].imag / (2 * math.pi * 1e3) > hf[1].imag / (2 * math.pi * 1e8)


@pytest.mark.parametrize("solve", SOLVERS)
def test_slot_raises_inductance_monotonically(solve):
    """test_solver.py:69-76."""
    L = [solve(synth.microstrip(slot=s), 1e8)[1].imag for s in (0.0, 6.0, 12.0)]
    assert L[0] < L[1] < L[2]


@pytest.mark.parametrize("solve", SOLVERS)
def test_split_from_edge_turns_the_loop_into_the_board_plane(solve):
    """test_solver.py:79-82: a cut from the edge makes the return go around it: the moment's z component
    (a loop in the board plane) dominates."""
    I_x, Z, m = solve(synth.microstrip(edge_split=True), 1e8)
    assert abs(m[2]) > 2 * abs(m[1])


def test_fully_cut_plane_is_refused():
    """test_solver.py:85-88: driver and receiver on separate pieces of copper."""
    b = synth.microstrip(full_cut=True)
    with pytest.raises(po.OracleSolverError):
        oracle_routes(oracle_stack(b), b)
    with pytest.raises(gs.SolverError):
        gs.from_board(b, _device=False)
