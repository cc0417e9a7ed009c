"""Parity of the CUDA path with the FP64 oracle on seeded boards drawn like the uneven-batch workload (2-6
plane layers, polygon cut-outs, stitching vias, non-square rasters) and on a six-layer stack with a slot on
every layer (the largest instance's shape), at sizes the oracle solves in seconds.  Needs a GPU."""
import numpy as np
import pytest

from groundtruth_gb300 import stack as gs, synth
from test_oracle_golden import oracle_routes, oracle_stack

pytestmark = pytest.mark.gpu
BOARDS = [("random", 31), ("random", 32), ("random", 33), ("random", 34), ("six_sheet", 21)]


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module", params=BOARDS, ids=[f"{k}{s}" for k, s in BOARDS])
def case(request):
    kind, seed = request.param
    board = synth.six_sheet(seed) if kind == "six_sheet" else synth.random_board(seed)
    ost = oracle_stack(board)
    oroutes = oracle_routes(ost, board)
    st, routes = gs.from_board(board)
    return board, ost, oroutes, st, routes


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_solves_match_oracle(case, precision):
    board, ost, oroutes, st, routes = case
    sols = gs.solve_many(routes, list(board.freqs), tol=board.tol, precision=precision)
    for k, per in enumerate(sols):
        for q, sol in enumerate(per):
            ref = oroutes[k].solve(float(board.freqs[q]), tol=board.tol)
            Ib = ref["x"][: ost.nb]
            assert rel(sol.state_for(st)[: st.ns], Ib[: ost.ns]) < 1e-7
            assert abs(sol.Z_loop - ref["Z_loop"]) <= 1e-8 * abs(ref["Z_loop"]), (k, q, sol.Z_loop, ref["Z_loop"])
            assert sol.residual <= board.tol


def test_six_sheet_column_pass_with_more_rows_than_threads():
    """Six sheets on a 600-row raster: the column FFTs (P0 = 1536) need 6 x 192 threads per column, more than a
    block holds, so the column pass transforms its rows in slots (the largest instance's 2048-point columns
    do the same).  The FP64 and FP32 L_p products against the oracle's."""
    from groundtruth_gb300 import native
    nx, ny, d, t = 600, 12, 0.3e-3, 35e-6
    layers = [synth._full_layer(f"L{k}", -k * 0.4e-3, t, nx, ny, d) for k in range(6)]
    pts = [(20 * d, 6 * d), (580 * d, 6 * d)]
    net = synth.Net(synth._segments(pts, 0.15e-3 + t, 0.5 * t, 0.15e-3), (0, 20, 6), (0, 580, 6))
    board = synth.Board("thin_six", d, nx, ny, layers, nets=[net], freqs=np.array([1e7]))
    ost = oracle_stack(board)
    st, routes = gs.from_board(board)
    obj, k = st.factorise([1e7])[0]
    rng = np.random.default_rng(9)
    I = rng.standard_normal(st.ns) + 1j * rng.standard_normal(st.ns)
    ref = ost.Lp_matvec(I)
    x = np.zeros(st.handle.n_compact, complex)
    x[: st.ns] = I
    # FP64 rounding of 1536- and 24-point transforms of random currents over six sheets (4.9e-12 measured)
    assert rel(native.apply(st.handle, obj, "lp", x, k, "fp64")[0][: st.ns], ref) < 1e-11
    assert rel(native.apply(st.handle, obj, "lp", x, k, "fp32")[0][: st.ns], ref) < 1e-5
