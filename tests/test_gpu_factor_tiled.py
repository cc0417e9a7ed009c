"""The blocked multi-CTA elimination of large fronts (factor.cu, tiled_*_kernel) against the reference's
preconditioner and against the one-CTA rank-1 elimination.  GT_TILED_NF, read when a geometry is made, sets the
front size from which the blocked path is taken: 1 sends every front through it (fronts smaller than one
32-column block, fronts without boundary rows, the root), a large value none.  Needs a GPU."""
import numpy as np
import pytest

from groundtruth_gb300 import native, stack as gs, synth
from test_oracle_golden import load

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _stack(board, tiled_nf, monkeypatch):
    monkeypatch.setenv("GT_TILED_NF", str(tiled_nf))
    return gs.from_board(board)


@pytest.mark.parametrize("name", ["small_pair", "small_stack3", "plain_plane", "faces_stack3_sheet"])
@pytest.mark.parametrize("tiled_nf", [1, 24])
def test_blocked_fronts_match_the_reference_preconditioner(name, tiled_nf, monkeypatch):
    z, board = load(name)
    st, routes = _stack(board, tiled_nf, monkeypatch)
    obj, k = st.factorise([float(z["op_f"])])[0]
    y = native.apply(st.handle, obj, "precond", z["prod_x"], k, "fp64")[0]
    assert rel(y, z["prod_precond"]) < 1e-9


@pytest.mark.parametrize("name", ["small_pair", "small_stack3"])
def test_blocked_fronts_solve_like_the_reference(name, monkeypatch):
    z, board = load(name)
    st, routes = _stack(board, 1, monkeypatch)
    sols = gs.solve_many(routes, list(board.freqs), tol=board.tol, precision="mixed")
    for kk, per in enumerate(sols):
        for q, sol in enumerate(per):
            Zr = complex(z[f"Z{kk}_{q}"])
            assert abs(sol.Z_loop - Zr) <= 1e-8 * abs(Zr), (kk, q, sol.Z_loop, Zr)
            assert rel(sol.state_for(st)[: st.ns], z[f"x{kk}_{q}"][: st.ns]) < 1e-7
            assert sol.residual <= board.tol


def test_blocked_and_rank1_elimination_agree_on_large_fronts(monkeypatch):
    """A board whose top fronts have 400-600 rows: its preconditioner with the blocked path (default) and
    with every front on the rank-1 kernel agree to FP64 rounding."""
    board = synth.uneven_board(21)
    f = float(board.freqs[len(board.freqs) // 2])
    rng = np.random.default_rng(3)
    out = []
    for tiled_nf in (256, 1 << 30):
        st, routes = _stack(board, tiled_nf, monkeypatch)
        assert max(st.sym.nown + st.sym.nbnd) >= 400
        n = st.handle.n_compact
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n) if not out else x
        obj, k = st.factorise([f])[0]
        out.append(native.apply(st.handle, obj, "precond", x, k, "fp64")[0])
    assert rel(out[0], out[1]) < 1e-11
