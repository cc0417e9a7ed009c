"""Derived stacks on the device (gt_operators_derive: the base's factor panels plus the Woodbury update of the
added branches) against the reference's own derived-stack outputs (tests/golden/small_pair_derived.npz) and the
oracle.  Needs a GPU."""
import numpy as np
import pytest

from groundtruth_gb300 import native, stack as gs, synth
from oracle import peec_oracle as po
from test_derived_stacks import branches_of, extra_of
from test_oracle_golden import load, oracle_routes, oracle_stack

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def case():
    z, board = load("small_pair_derived")
    extra = extra_of(z)
    st, routes = gs.from_board(board)
    dst = st.with_branches(branches_of(extra))
    return z, board, extra, st, routes, dst


def test_derived_geometry_and_operators(case):
    z, board, extra, st, routes, dst = case
    assert dst._base is st and dst.n_lowrank == len(extra)
    (obj, k), = dst.factorise([float(board.freqs[0])])
    assert obj.base is st.factorise([float(board.freqs[0])])[0][0]
    # a geometry with a low-rank tail cannot be factorised on its own
    with pytest.raises(ValueError):
        native.Operators(dst.handle, [1e8], [dst._freq_tables(1e8)])


def test_derived_products_match_reference(case):
    z, board, extra, st, routes, dst = case
    (obj, k), = dst.factorise([float(board.freqs[0])])
    y = native.apply(dst.handle, obj, "matvec", z["prod_x"], k, "fp64")[0]
    assert rel(y, z["prod_matvec"]) < 1e-12
    y = native.apply(dst.handle, obj, "precond", z["prod_x"], k, "fp64")[0]
    assert rel(y, z["prod_precond"]) < 1e-9
    y32 = native.apply(dst.handle, obj, "precond", z["prod_x"], k, "fp32")[0]
    assert rel(y32, z["prod_precond"]) < 1e-3


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_derived_solves_match_reference(case, precision):
    z, board, extra, st, routes, dst = case
    droutes = [r.on(dst) for r in routes]
    sols = gs.solve_many(droutes, list(board.freqs), tol=board.tol, precision=precision)
    for k, per in enumerate(sols):
        for q, sol in enumerate(per):
            ref = z[f"Z{k}_{q}"]
            assert abs(sol.Z_loop - ref) <= 1e-8 * abs(ref), (k, q, sol.Z_loop, ref)
            x = sol.state_for(dst)
            assert rel(x[: dst.nb], z[f"x{k}_{q}"][: dst.nb]) < 1e-7
            assert sol.residual <= board.tol


def test_warm_start_from_base_solution(case):
    """The what-if loop: the base's solution, mapped onto the derived stack with the new branches at zero,
    starts the derived solve (suggest.py:318-325); same answer, fewer iterations."""
    z, board, extra, st, routes, dst = case
    f = float(board.freqs[1])
    base = routes[0].solve(f, tol=board.tol)
    rd = routes[0].on(dst)
    cold = rd.solve(f, tol=board.tol)
    warm = rd.solve(f, guess=[dst.map_state(base.state_for(st), st)], tol=board.tol)
    assert abs(warm.Z_loop - z["Z0_1"]) <= 1e-8 * abs(z["Z0_1"])
    assert warm.iterations < cold.iterations


def test_derived_of_derived_matches_whole_stack_oracle(case):
    """Two edits in a row derive from the first base with both edits' branches; the solve equals the oracle's
    solve of the whole stack factorised afresh."""
    z, board, extra, st, routes, dst = case
    more = synth.what_if_branches(board, seed=12, n_via=2, n_part=0)
    d2 = dst.with_branches(branches_of(more))
    assert d2._base is st and d2.n_lowrank == len(extra) + len(more)
    whole = synth.Board.from_arrays(board.to_arrays())
    whole.branches = list(board.branches) + list(extra) + list(more)
    ost = oracle_stack(whole)
    assert ost.nb == d2.nb
    oroute = oracle_routes(ost, whole)[1]
    f = float(board.freqs[2])
    sol = routes[1].on(d2).solve(f, tol=board.tol)
    ref = oroute.solve(f, tol=board.tol)
    assert abs(sol.Z_loop - ref["Z_loop"]) <= 1e-8 * abs(ref["Z_loop"])


def test_what_if_service(case):
    """The what-if service (whatif.WhatIf): a solved base, one edit on two nets at two frequencies, warm
    started from the base's solutions; the same answers as the reference's derived stack."""
    from groundtruth_gb300 import whatif
    z, board, extra, st, routes, dst = case
    wi = whatif.WhatIf(st, routes, board.freqs, tol=board.tol)
    wi.baseline()
    res = wi.evaluate(branches_of(extra), [0, 1], [float(board.freqs[1]), float(board.freqs[2])])
    for (k, f), sol in res.solutions.items():
        q = [float(v) for v in board.freqs].index(f)
        ref = z[f"Z{k}_{q}"]
        assert abs(sol.Z_loop - ref) <= 1e-8 * abs(ref), (k, q)
        assert sol.residual <= board.tol
    assert res.parts["cold_redo"] == 0


@pytest.mark.parametrize("method", ["bordered", "derived"])
def test_what_if_methods_agree_with_oracle_whole_stack(case, method):
    """Both ways of answering an edit give the whole edited board's solution (oracle, factorised afresh)."""
    from groundtruth_gb300 import whatif
    z, board, extra, st, routes, dst = case
    more = synth.what_if_branches(board, seed=13, n_via=3, n_part=1)
    whole = synth.Board.from_arrays(board.to_arrays())
    whole.branches = list(board.branches) + list(more)
    ost = oracle_stack(whole)
    oroutes = oracle_routes(ost, whole)
    wi = whatif.WhatIf(st, routes, board.freqs, tol=board.tol, method=method)
    wi.baseline()
    res = wi.evaluate(branches_of(more), [0, 1], [float(f) for f in board.freqs])
    for (k, f), sol in res.solutions.items():
        ref = oroutes[k].solve(f, tol=board.tol)
        assert abs(sol.Z_loop - ref["Z_loop"]) <= 1e-8 * abs(ref["Z_loop"]), (method, k, f)
        assert sol.residual <= board.tol
    if method == "bordered":
        assert res.parts["border_columns"] == len(more) * len(board.freqs)


@pytest.mark.parametrize("method", ["bordered", "derived"])
def test_moved_part_matches_oracle(case, method):
    """A decoupling part moved elsewhere (removed and added) answered on the device equals the oracle's solve of
    the board with the part moved."""
    from groundtruth_gb300 import whatif
    z, board, extra, st, routes, dst = case
    decap = board.branches[0]
    moved = synth.BranchSpec((0, 30, 10), (1, 30, 10), decap.R, decap.L, decap.C, decap.kind, decap.radius)
    whole = synth.Board.from_arrays(board.to_arrays())
    whole.branches = [moved] + list(board.branches[1:])
    oroutes = oracle_routes(oracle_stack(whole), whole)
    wi = whatif.WhatIf(st, routes, board.freqs, tol=board.tol, method=method)
    wi.baseline()
    f = float(board.freqs[1])
    res = wi.evaluate(branches_of([moved]), [0, 1], [f], remove=[0])
    for k in (0, 1):
        ref = oroutes[k].solve(f, tol=board.tol)
        assert abs(res.solutions[(k, f)].Z_loop - ref["Z_loop"]) <= 1e-8 * abs(ref["Z_loop"]), (method, k)


@pytest.mark.parametrize("name", ["necked_pair", "faces_stack3_sheet", "necked_faces"])
@pytest.mark.parametrize("method", ["bordered", "derived"])
def test_edits_on_narrow_and_face_sheet_boards(name, method):
    """Added vias and a part on boards with narrow strips and face sheets, both ways, against the oracle's
    solve of the whole edited board."""
    from groundtruth_gb300 import whatif
    z, board = load(name)
    st, routes = gs.from_board(board)
    more = synth.what_if_branches(board, seed=5, n_via=2, n_part=1)
    whole = synth.Board.from_arrays(board.to_arrays())
    whole.branches = list(board.branches) + list(more)
    oroutes = oracle_routes(oracle_stack(whole), whole)
    wi = whatif.WhatIf(st, routes, board.freqs, tol=board.tol, method=method)
    wi.baseline()
    f = float(board.freqs[-1])
    res = wi.evaluate(branches_of(more), [0], [f])
    ref = oroutes[0].solve(f, tol=board.tol)
    assert abs(res.solutions[(0, f)].Z_loop - ref["Z_loop"]) <= 1e-8 * abs(ref["Z_loop"]), (name, method)
