"""The reference's analytic known-answer cases for this solve (tests/test_solver.py:31-88 of GroundTruth),
restated on a 40 x 20 mm plane under a microstrip (synth.microstrip): the strip kernel's symmetry and self term,
the return current under the trace against image theory, the loop inductance against Wheeler's formula and
the moment against the loop's area, current spreading at low frequency, a slot's monotonic effect, a cut from
the edge turning the loop into the board plane, a fully cut plane refused, a plane pair's inductance per
length (tests/test_plane_pair.py:70-81), a track's resistance from its rasterised copper
(tests/test_track_width.py:91-157), and the reciprocity of two loops' mutual impedance.  Each runs on the oracle (CPU)
and, marked gpu, through the CUDA library."""
import math
from pathlib import Path

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


@pytest.mark.parametrize("solve", SOLVERS)
def test_plane_pair_inductance_per_length(solve):
    """test_plane_pair.py:70-81: a parallel-plate line 10 mm wide, 0.2 mm between its 35 um foils, shorted at
    its far end; the difference of a 40 mm and a 20 mm line is the inductance of 20 mm of line alone.  At 1 MHz
    (skin depth 66 um > t) mu0 (h + 2t/3) / w, at 100 MHz (6.6 um) mu0 (h + delta) / w, each within -6 % / +3 %
    (the field fringing past the edges lowers it), and the high-frequency value the lower one."""
    mu0, sigma, h, w, t = 4e-7 * math.pi, 5.8e7, 0.2e-3, 10e-3, 35e-6
    L = {ln: [] for ln in (20.0, 40.0)}
    for ln in L:
        b = synth.plane_pair_line(ln)
        for f in b.freqs:
            L[ln].append(solve(b, f)[1].imag / (2 * math.pi * f))
    per = [(l40 - l20) / 20e-3 for l20, l40 in zip(L[20.0], L[40.0])]
    low = mu0 * (h + 2 * t / 3) / w
    high = mu0 * (h + 1 / math.sqrt(math.pi * 1e8 * mu0 * sigma)) / w
    assert 0.94 * low < per[0] < 1.03 * low, (per[0], low)
    assert 0.94 * high < per[1] < 1.03 * high, (per[1], high)
    assert per[1] < per[0]


@pytest.mark.parametrize("name", list(synth.KNOWN_BOARDS))
@pytest.mark.parametrize("solve", SOLVERS)
def test_known_answer_boards_match_the_reference(solve, name):
    """The known-answer boards' loop impedances and moments against the reference's own solves of the same
    boards (tests/golden/known_answers.npz), both at rtol 1e-10: Z_loop within 1e-8, m within 1e-6."""
    ref = np.load(Path(__file__).resolve().parent / "golden" / "known_answers.npz")
    board = synth.KNOWN_BOARDS[name]()
    board.tol = 1e-10
    assert np.array_equal(ref[f"{name}_freqs"], board.freqs)
    for q, f in enumerate(board.freqs):
        _, Z, m = solve(board, float(f))
        Zr, mr = complex(ref[f"{name}_Z{q}"]), ref[f"{name}_m{q}"]
        assert abs(Z - Zr) <= 1e-8 * abs(Zr), (name, f, Z, Zr)
        assert np.linalg.norm(m - mr) <= 1e-6 * np.linalg.norm(mr), (name, f)


@pytest.mark.parametrize("width, angle, dy, tol", [(0.4, 0.0, 0.0, 0.01), (0.1, 0.0, 0.03, 0.01),
                                                    (0.05, 0.0, 0.06, 0.01), (0.4, 30.0, 0.0, 0.015),
                                                    (0.15, 45.0, 0.0, 0.015), (0.1, 30.0, 0.0, 0.015)])
@pytest.mark.parametrize("solve", SOLVERS)
def test_a_track_has_the_resistance_of_its_cross_section(solve, width, angle, dy, tol):
    """test_track_width.py:91-157 (TW-1, TW-3): a track rasterised from its copper with exact widths (0.5 mm
    pitch, 0.125 mm sub-grid), 0.4, 0.1 or 0.05 mm wide, on or off the grid's rows, straight or at 30 or 45
    degrees (a staircase of x and y strips, each as wide as the border its copper crosses), has the resistance
    per length 1 / (sigma w t): the difference of a 40 and a 20 mm track's DC resistances over 20 mm, within
    1 % (straight) / 1.5 % (at an angle)."""
    r = [solve(synth.track_rail(length, width, angle, dy), 0.0)[1].real for length in (20.0, 40.0)]
    assert (r[1] - r[0]) / 0.020 == pytest.approx(1 / (5.8e7 * width * 1e-3 * 35e-6), rel=tol)


def _two_loops_oracle(board, f):
    st = oracle_stack(board)
    rs = oracle_routes(st, board)
    net = board.nets[0]
    other = rs[1] if len(rs) > 1 else po.OracleRoute(st, [], net.driver, net.receiver)
    out = []
    for r in (rs[0], other):
        Ib, V, *_ = st.solve(f, r.rhs_top(f), r.J(), tol=1e-12)
        out.append((r.psi, r.J(), Ib, V))
    return out


def _two_loops_device(board, f):
    st, routes = gs.from_board(board)
    net = board.nets[0]
    rs = [routes[0], routes[1] if len(routes) > 1 else gs.RouteExcitation(st, [], net.driver, net.receiver)]
    res = st.solve_batch([f, f], [r.rhs_top(f) for r in rs], [r.J() for r in rs], tol=1e-10)
    return [(r.psi, r.J(), o[0], o[1]) for r, o in zip(rs, res)]


@pytest.mark.parametrize("name", ["small_pair", "necked_pair", "necked_faces", "six_sheet"])
@pytest.mark.parametrize("solve", [pytest.param(_two_loops_oracle, id="oracle"),
                                   pytest.param(_two_loops_device, id="gpu", marks=pytest.mark.gpu)])
def test_mutual_impedance_is_reciprocal(solve, name):
    """Reciprocity, a property of the system at any size (its matrix is complex symmetric: the partial
    inductances, the narrow strips' mutual corrections and the face couplings are): the plane's part of the
    mutual impedance of two loops, j omega psi_a . I_b + J_a . V_b, is the same both ways.  The loops are the
    board's first two nets, or its first net and a port at the same return nodes without the trace; with plane
    pairs, narrow strips, face sheets and six layers."""
    board = getattr(synth, name)()
    for f in board.freqs[:2]:
        w = 2 * math.pi * f
        loops = solve(board, float(f))
        z = [[1j * w * np.dot(a[0], b[2]) + a[1] @ b[3] for b in loops] for a in loops]
        scale = math.sqrt(abs(z[0][0] * z[1][1]))
        assert abs(z[0][1]) > 1e-3 * scale
        assert abs(z[0][1] - z[1][0]) <= 1e-7 * scale, (name, f)


def _tape_integral(length, wa, wb, axial, lateral, dz):
    """The two tapes' mutual inductance by adaptive quadrature of the width-difference integral (independent of
    the panel rules under test)."""
    from scipy.integrate import quad

    def f(v):
        over = min(0.5 * wa, v + 0.5 * wb) - max(-0.5 * wa, v - 0.5 * wb)
        return max(over, 0.0) * float(greens.filament_mutual(length, axial, math.hypot(lateral + v, dz)))
    h, k = 0.5 * (wa + wb), 0.5 * abs(wa - wb)
    pts = sorted({-h, -k, k, h} | ({-lateral} if -h < -lateral < h else set()))
    return sum(quad(f, p, q, limit=400, epsabs=0, epsrel=1e-12)[0] for p, q in zip(pts[:-1], pts[1:]) if q > p) / (wa * wb)


@pytest.mark.parametrize("case", [(1, 1, 0, 0, 0), (1, 1, 1, 0, 0), (1, 1, 0, 1, 0), (1, 1, 0, 0, 0.05),
                                  (1, 1, 1, 1, 0.02), (0.3, 1, 0, 0.6, 0), (0.1, 0.7, 2, 0.4, 0.001)])
def test_tape_mutual_is_the_integral(case):
    """test_numerics_audit.py:311-322: the tapes' near-field mutual and the strip's self term equal the integral
    to 1e-9 (host setup and oracle)."""
    d = 0.5e-3
    wa, wb, a, lat, dz = (v * d for v in case)
    ref = _tape_integral(d, wa, wb, a, lat, dz)
    for mod in (greens, po):
        assert mod.tape_mutual(d, wa, wb, a, lat, dz) == pytest.approx(ref, rel=1e-9)
        assert float(mod.strip_self_numeric(d, d)) == pytest.approx(_tape_integral(d, d, d, 0, 0, 0), rel=1e-9)


@pytest.mark.parametrize("ratio, tol", [(2.0, 0.006), (10.0, 0.002), (20.0, 0.002)])
def test_plane_pair_sheet_inductance_is_mu0_dz(ratio, tol):
    """test_numerics_audit.py:325-339: opposite uniform currents on two planes dz apart have mu0 dz of loop
    inductance per square, 2 sum(K(0) - K(dz)) over a 41 x 41 plane, however thin the gap."""
    d, n = 0.5e-3, 41
    dz = d / ratio
    for mod in (greens, po):
        sheet = 2 * (mod.strip_kernel(n, n, d, 0.0) - mod.strip_kernel(n, n, d, dz)).sum()
        assert sheet == pytest.approx(4e-7 * math.pi * dz, rel=tol)


@pytest.mark.parametrize("t_um", [18.0, 35.0, 70.0, 105.0, 210.0])
def test_slab_impedance_is_the_coth_form(t_um):
    """test_plane_pair.py:84-106: the one-face slab (1 + j)/(sigma delta) coth((1 + j) t/delta) from 1 kHz to
    20 GHz within 1e-5, its half-space limit beyond t/delta = 30 within 1e-9."""
    sigma, mu0 = 5.8e7, 4e-7 * math.pi
    t = t_um * 1e-6
    for f in np.logspace(3, np.log10(2e10), 60):
        delta = 1 / math.sqrt(math.pi * f * mu0 * sigma)
        u = (1 + 1j) * t / delta
        if abs(u) < 1e-3:
            ref = (1 + u ** 2 / 3 - u ** 4 / 45 + 2 * u ** 6 / 945) / (sigma * t)
        else:
            ref = u * (1 + np.exp(-2 * u)) / (1 - np.exp(-2 * u)) / (sigma * t)
        for mod in (greens, po):
            z = complex(mod.slab_impedance(t, f, sigma))
            assert abs(z.real / ref.real - 1) < 1e-5 and abs(z.imag / ref.imag - 1) < 1e-5, (t_um, f)
            if t / delta > 30:
                assert abs(z / ((1 + 1j) / (sigma * delta)) - 1) < 1e-9


def test_oracle_gmres_solves_like_a_direct_solve():
    """test_speed.py:18-28: restarted GMRES reaches the direct solution to 1e-8 across restarts, and stops at its
    iteration budget with the best solution so far."""
    rng = np.random.default_rng(1)
    n = 60
    A = np.eye(n) * 4 + rng.standard_normal((n, n)) / np.sqrt(n) + 1j * rng.standard_normal((n, n)) / np.sqrt(n)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    x, its, ok = po.gmres(lambda v: A @ v, b, 1e-10, restart=15, max_cycles=40)
    assert ok and its > 15
    assert np.linalg.norm(x - np.linalg.solve(A, b)) < 1e-8 * np.linalg.norm(x)
    D = np.arange(1.0, 201.0)                   # needs ~200 iterations: stopped at its budget, the best so far
    x, its, ok = po.gmres(lambda v: D * v, np.ones(200, complex), 1e-10, max_its=7)
    assert not ok and its == 7 and np.linalg.norm(D * x - 1) < np.sqrt(200)


def test_oracle_gmres_goes_on_while_its_residual_falls():
    """test_speed.py:31-45: restarts beyond max_cycles while each still lowers the residual, none once it
    stalls (GMRES(4) on a cyclic shift makes no progress)."""
    rng = np.random.default_rng(2)
    n = 120
    A = np.eye(n) * 3 + rng.standard_normal((n, n)) / np.sqrt(n)
    b = rng.standard_normal(n).astype(complex)
    _, its, ok = po.gmres(lambda v: A @ v, b, 1e-10, restart=4, max_cycles=3)
    assert not ok and its == 12
    x, its, ok = po.gmres(lambda v: A @ v, b, 1e-10, restart=4, max_cycles=3, extra_cycles=40)
    assert ok and its > 12 and np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)
    P = np.roll(np.eye(n), 1, axis=0)
    _, its, ok = po.gmres(lambda v: P @ v, np.eye(n)[0].astype(complex), 1e-10, restart=4, max_cycles=2,
                          extra_cycles=40)
    assert not ok and its <= 3 * 4


def _dc_drop(board):
    """The plane's DC drop between the receiver and driver nodes by a direct solve of its resistive network
    (every strip a square of sheet resistance 1/(sigma t) between its nodes; GroundTruth's DC sheet reference,
    tests/refsolvers.py:96-153, on the solver's own grid)."""
    import scipy.sparse as sp
    from scipy.sparse.linalg import spsolve
    st = gs.from_board(board, _device=False)[0]
    g = st.sigma * st.ts[0]
    a, b = st.top.a_nodes[: st.ns], st.top.b_nodes[: st.ns]
    n = st.n_nodes
    L = sp.coo_matrix((np.concatenate([np.full(st.ns, g)] * 2 + [np.full(st.ns, -g)] * 2),
                       (np.concatenate([a, b, a, b]), np.concatenate([a, b, b, a]))), shape=(n, n)).tocsr()
    net = board.nets[0]
    drv, rcv = int(st.nid[net.driver]), int(st.nid[net.receiver])
    J = np.zeros(n)
    J[drv], J[rcv] = -1.0, 1.0
    keep = np.flatnonzero(st.keep)
    V = np.zeros(n)
    V[keep] = spsolve(L[keep][:, keep].tocsc(), J[keep])
    return V[rcv] - V[drv]


@pytest.mark.parametrize("solve", SOLVERS)
def test_dc_limit_is_the_resistive_sheet(solve):
    """At 0 Hz the solve is the plane's resistive network: the loop impedance's plane part (the injections'
    potential difference) equals a direct solve of the sheet's conductance Laplacian."""
    b = synth.microstrip(f=(0.0,))
    b.tol = 1e-10
    I_x, Z, m = solve(b, 0.0)
    seg = b.nets[0].segments
    r_trace = greens.trace_resistance(seg, 0.0, b.sigma, b.nets[0].trace_t)
    assert Z.imag == pytest.approx(0.0, abs=1e-12)
    assert Z.real - r_trace == pytest.approx(_dc_drop(b), rel=1e-8)


def _solution_oracle(board, f, route=None):
    """The oracle's solve of a board's first net (or `route` on the host stack) as the mirror's Solution."""
    st, routes = gs.from_board(board, _device=False)
    r = route(st) if route is not None else routes[0]
    ost = oracle_stack(board)
    Ib, V, its, x = ost.solve(f, r.rhs_top(f), r.J(), tol=board.tol)
    return r.solution(f, Ib, V, its)


def _solution_device(board, f, route=None):
    st, routes = gs.from_board(board)
    r = route(st) if route is not None else routes[0]
    return r.solve(f, tol=board.tol)


SOLUTIONS = [pytest.param(_solution_oracle, id="oracle"),
             pytest.param(_solution_device, id="gpu", marks=pytest.mark.gpu)]


@pytest.mark.parametrize("solve", SOLUTIONS)
def test_the_return_current_flows_back_under_the_trace(solve):
    """test_vectors.py:42-54: at 100 MHz the plane's current at the dominant phase flows -x right under the +x
    trace, sums across the plane to the whole signal current back, and carries the full magnitude there; the
    same currents turned by any phase give the same vectors (test_vectors.py:57-68)."""
    import dataclasses
    b = synth.microstrip()
    b.tol = 1e-8
    sol = solve(b, 1e8)
    d_mm = b.d * 1e3
    kx, ky = sol.sheet_vectors(0, d_mm)
    i, j = 80, 40
    assert kx[i, j] < 0 and abs(ky[i, j]) < 0.01 * abs(kx[i, j])
    assert float(np.sum(kx[i, :]) * b.d) == pytest.approx(-1.0, abs=0.02)
    y = np.arange(b.ny) * b.d - 10e-3
    near = np.abs(y) < 3 * H
    assert np.allclose(np.hypot(kx, ky)[i, near], sol.sheet_current(0, d_mm)[i, near], rtol=0.01)
    for theta in (0.6, -1.2):
        turned = dataclasses.replace(sol, I_x=sol.I_x * np.exp(1j * theta), I_y=sol.I_y * np.exp(1j * theta))
        tx, ty = turned.sheet_vectors(0, d_mm)
        assert np.allclose(tx, kx, atol=1e-9 * np.abs(kx).max()) and np.allclose(ty, ky, atol=1e-9 * np.abs(kx).max())


@pytest.mark.parametrize("solve", SOLUTIONS)
def test_a_node_where_current_enters_reads_its_strips_heat(solve):
    """test_density_maps.py:106-123: 1 A into the middle of a 10 x 10 mm plane (0.25 mm cells), out at four nodes
    near its corners: the mean of the middle node's four strips cancels (0), the heat-consistent density (copper)
    is sqrt(1/8)/d there (four strips of 0.25 A), highest where the current enters, and away from the feed both
    definitions agree."""
    n, d_mm = 41, 0.25
    node = np.ones((n, n), bool)
    layer = synth.Layer("F", 0.0, 35e-6, node, np.ones((n - 1, n), bool), np.ones((n, n - 1), bool))
    board = synth.Board("feed", d_mm * 1e-3, n, n, [layer], freqs=np.array([10.0]), tol=1e-10)
    c = (0, n // 2, n // 2)
    out = [(0, 2, 2), (0, n - 3, 2), (0, 2, n - 3), (0, n - 3, n - 3)]
    route = lambda st: gs.RouteExcitation(st, [], injections=[(c, 1.0)] + [(k, -0.25) for k in out])  # noqa: E731
    sol = solve(board, 10.0, route)
    i, j = c[1], c[2]
    assert sol.sheet_current(0, d_mm)[i, j] == pytest.approx(0.0, abs=1e-6)
    heat = sol.sheet_current(0, d_mm, True)
    assert heat[i, j] == pytest.approx(math.sqrt(1 / 8) / (d_mm * 1e-3), rel=1e-6)
    assert heat[i, j] > heat[i + 1, j] > heat[i + 2, j]
    assert heat[i, 5] == pytest.approx(sol.sheet_current(0, d_mm)[i, 5], rel=0.02)


@pytest.mark.parametrize("name", ["small_pair", "necked_faces", "routed_pair"])
def test_a_solutions_state_is_rebuilt_exactly_from_its_currents_and_potentials(name):
    """test_solver.py:271-300: Solution.state_for rebuilds the solver's unknown vector from the solution's strip,
    capacitance, branch (and face-pair) currents and its node potentials, every number the same."""
    from test_oracle_golden import load
    z, board = load(name)
    st, routes = gs.from_board(board, _device=False)
    ost = oracle_stack(board)
    f = float(board.freqs[0])
    r = routes[0]
    Ib, V, its, x = ost.solve(f, r.rhs_top(f), r.J(), tol=1e-8)
    sol = r.solution(f, Ib, V, its)
    assert np.array_equal(sol.state_for(st), x)
