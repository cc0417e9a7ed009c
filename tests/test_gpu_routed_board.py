"""A plane pair rasterised from polygons (raster.build_layer, the reference's build_grid at sub-grid 4, with
exact widths: synth.routed_pair) solved through the CUDA library against the reference's own solves of it
(tests/golden/routed_pair.npz).  Needs a GPU."""
import numpy as np
import pytest

from groundtruth_gb300 import native, stack as gs
from test_oracle_golden import load

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_routed_board_products_and_solves():
    z, board = load("routed_pair")
    st, routes = gs.from_board(board)
    obj, k = st.factorise([float(z["op_f"])])[0]
    assert rel(native.apply(st.handle, obj, "matvec", z["prod_x"], k, "fp64")[0], z["prod_matvec"]) < 1e-12
    assert rel(native.apply(st.handle, obj, "precond", z["prod_x"], k, "fp64")[0], z["prod_precond"]) < 1e-9
    sols = gs.solve_many(routes, list(board.freqs), tol=board.tol)
    for kk, per in enumerate(sols):
        for q, sol in enumerate(per):
            Zr = complex(z[f"Z{kk}_{q}"])
            assert abs(sol.Z_loop - Zr) <= 1e-8 * abs(Zr), (kk, q)
            assert rel(sol.m, z[f"m{kk}_{q}"]) < 1e-7
            assert sol.residual <= board.tol
