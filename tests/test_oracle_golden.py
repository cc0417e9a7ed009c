"""The CPU oracle against the reference's own outputs (tests/golden/*.npz, made by make_golden.py).

These pins are what makes the oracle trustworthy as the GPU build's checker: the restated topology and
index work must be bit-exact, the kernels, operators and products equal to FP64 rounding, and the solves
equal to the GMRES tolerance."""
from pathlib import Path

import numpy as np
import pytest

from groundtruth_gb300 import synth
from oracle import peec_oracle as po

GOLD = Path(__file__).resolve().parent / "golden"
CASES = ["small_pair", "small_stack3", "plain_plane", "necked_pair", "faces_stack3_diag", "faces_stack3_sheet",
         "necked_faces", "routed_pair"]


def load(name):
    z = np.load(GOLD / f"{name}.npz", allow_pickle=False)
    board = synth.Board.from_arrays({k[len("board_"):]: z[k] for k in z.files if k.startswith("board_")})
    return z, board


def oracle_stack(board):
    layers = [po.OLayer(l.z, l.thickness, l.node, l.xb, l.yb, l.widths, l.fill) for l in board.layers]
    pairs = [po.OPair(p.upper, p.lower, p.c_per_area, p.tan_delta) for p in board.pairs]
    branches = [po.OBranch(b.a, b.b, b.R, b.L, b.C, b.kind, b.radius) for b in board.branches]
    return po.OracleStack(layers, board.d, branches, pairs, board.sigma, board.precond, board.screen)


def oracle_routes(st, board):
    out = []
    for net in board.nets:
        trace = [po.OSegment(s[0:3].copy(), s[3:6].copy(), float(s[6]), float(s[7])) for s in net.segments]
        out.append(po.OracleRoute(st, trace, net.driver, net.receiver, net.trace_t))
    return out


@pytest.fixture(scope="module", params=CASES)
def case(request):
    z, board = load(request.param)
    st = oracle_stack(board)
    return request.param, z, board, st


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


def test_kernel_functions_match_reference():
    z = np.load(GOLD / "kernel_functions.npz")
    L, ax, rho = z["fm_args"]
    assert rel(po.filament_mutual(L, ax, rho), z["fm"]) < 1e-14
    got = np.array([po.tape_mutual(*a) for a in z["tape_args"]])
    assert rel(got, z["tape"]) < 1e-13
    assert rel(po.strip_self_numeric(1e-3, z["ssn_w"]), z["ssn"]) < 1e-14
    assert rel(po.skin_thickness(35e-6, z["sk_f"], 5.8e7), z["skin35"]) < 1e-14
    assert rel(po.slab_impedance(18e-6, z["sk_f"], 5.8e7), z["slab18"]) < 1e-14
    assert rel(po.slab_impedance(35e-6, z["sk_f"], 5.8e7), z["slab35"]) < 1e-14
    assert rel(po.strip_kernel(6, 5, 0.5e-3, 0.3e-3), z["strip_kernel_6x5"]) < 1e-14


def test_topology_is_bit_exact(case):
    name, z, board, st = case
    for k in ("xa", "ya", "nid", "keep", "a_nodes", "b_nodes", "full_label", "cond_label"):
        assert np.array_equal(getattr(st, k), z[k]), k
    assert (st.nb, st.ns, st.ncap, st.nbr) == (int(z["nb"]), int(z["ns"]), int(z["ncap"]), int(z["nbr"]))
    assert np.array_equal(st.cap, z["cap"])
    assert tuple(st.Px) == tuple(z["Px"]) and tuple(st.Py) == tuple(z["Py"])


def test_kernels_match_reference(case):
    name, z, board, st = case
    assert rel(st.Kq["x"], z["Kq_x"]) < 1e-13
    assert rel(st.Kq["y"], z["Kq_y"]) < 1e-13
    assert st.L_self == pytest.approx(float(z["L_self"]), rel=1e-14)
    if "B_x" in z.files:
        assert rel(st.B_x, z["B_x"]) < 1e-13 and rel(st.B_y, z["B_y"]) < 1e-13


def test_operator_and_products_match_reference(case):
    name, z, board, st = case
    op = st.operator(float(z["op_f"]))
    assert rel(op["R_strip"], z["op_R"]) < 1e-14
    assert rel(op["z_tail"], z["op_z"]) < 1e-14
    D = op["Dinv"].tocoo()
    import scipy.sparse as sp
    ref = sp.coo_matrix((z["op_Dinv"], tuple(z["op_Dinv_ij"])), shape=D.shape).tocsr()
    assert abs(op["Dinv"] - ref).max() <= 1e-13 * abs(ref).max()
    Sref = sp.coo_matrix((z["op_S"], tuple(z["op_S_ij"])), shape=op["S"].shape).tocsr()
    assert abs(op["S"] - Sref).max() <= 1e-13 * abs(Sref).max()
    x, I = z["prod_x"], z["prod_I"]
    assert rel(st.Lp_matvec(I), z["prod_Lp"]) < 1e-12
    assert rel(st.matvec(op, x), z["prod_matvec"]) < 1e-12
    assert rel(st.precond(op, x), z["prod_precond"]) < 1e-9


def test_coupling_and_solves_match_reference(case):
    name, z, board, st = case
    routes = oracle_routes(st, board)
    for k, r in enumerate(routes):
        assert rel(r.psi, z[f"psi{k}"]) < 1e-13
        assert r.L_trace == pytest.approx(float(z[f"Ltrace{k}"]), rel=1e-13)
        for q, f in enumerate(board.freqs):
            op = st.operator(float(f))
            sol = r.solve(float(f), tol=board.tol, restart=board.restart, op=op)
            # both sides stop at a backward error of tol: the forward difference is within a few cond x tol
            assert rel(sol["x"], z[f"x{k}_{q}"]) < 1e-7, (k, f)
            assert abs(sol["Z_loop"] - z[f"Z{k}_{q}"]) <= 1e-8 * abs(z[f"Z{k}_{q}"]), (k, f)
            assert rel(sol["m"], z[f"m{k}_{q}"]) < 1e-7
            assert abs(sol["its"] - int(z[f"its{k}_{q}"])) <= 2


@pytest.mark.parametrize("name", ["necked_pair", "routed_pair"])
def test_narrow_strip_corrections_match_reference(name):
    """Strips narrower than the pitch (peec.py:1732-1820): widths, resistance widths, the self-inductance
    change dL and the side-by-side mutual changes M_near equal the reference's."""
    import scipy.sparse as sp
    z, board = load(name)
    st = oracle_stack(board)
    assert np.array_equal(st.strip_width, z["strip_width"]) and np.array_equal(st.r_width, z["r_width"])
    assert (st.strip_width < 1).sum() > 0 and rel(st.dL, z["dL"]) < 1e-12
    ij = z["M_near_ij"]
    ref = sp.coo_matrix((z["M_near"], (ij[0], ij[1])), shape=(st.ns, st.ns)).tocsr()
    assert st.M_near.nnz == ref.nnz and abs(st.M_near - ref).max() <= 1e-12 * abs(ref).max()


@pytest.mark.parametrize("name", ["faces_stack3_diag", "faces_stack3_sheet"])
def test_face_sheets_match_reference(name):
    """Screened layers split into two face sheets (peec.py:1658-1716, 2186-2197): the sheets, their layers and
    heights, the twin strip pairs and the face coupling equal the reference's."""
    z, board = load(name)
    st = oracle_stack(board)
    assert st.n_sheets == int(z["n_sheets"]) and np.array_equal(st.sheet_layer, z["sheet_layer"])
    assert np.array_equal(st.tw_a, z["tw_a"]) and np.array_equal(st.tw_b, z["tw_b"])
    assert np.allclose(st.sheet_z, z["sheet_z"], rtol=0, atol=1e-15) and np.array_equal(st.sheet_t, z["sheet_t"])
    assert rel(st.twin_z(float(z["op_f"])), z["op_Z12"]) < 1e-13


@pytest.mark.parametrize("name", ["necked_pair_scaled", "faces_stack3_sheet_scaled"])
def test_resistance_scale_matches_reference(name):
    """PlaneStack.set_resistance_scale (peec.py:2199-2216): strips' and branches' resistances scaled, their
    internal inductance kept; the preconditioner then takes every position on its own."""
    z, board = load(name)
    st = oracle_stack(board)
    st.set_resistance_scale(z["r_scale"], z["branch_scale"])
    op = st.operator(float(z["op_f"]))
    assert rel(op["R_strip"], z["op_R"]) < 1e-14 and rel(op["z_tail"], z["op_z"]) < 1e-14
    assert rel(st.matvec(op, z["prod_x"]), z["prod_matvec"]) < 1e-12
    assert rel(st.precond(op, z["prod_x"]), z["prod_precond"]) < 1e-10
    ref = oracle_routes(st, board)[0].solve(float(board.freqs[1]), tol=board.tol)
    assert abs(ref["Z_loop"] - z["Z0_1"]) <= 1e-8 * abs(z["Z0_1"])


def test_branch_impedances_match_reference():
    """via_impedance / track_impedance (peec.py:1061-1090): the product's restatement at a few sizes and
    frequencies equals the reference's."""
    from groundtruth_gb300 import stack as gs
    z = np.load(GOLD / "kernel_functions.npz")
    f = z["bf_f"]
    for (l, dr, fl), ref in zip(z["bf_via_args"], z["bf_via"]):
        got = np.array([gs.via_impedance(l, dr, filled=bool(fl))(x) for x in f])
        assert rel(got, ref) < 1e-13
    for (l, w, t), ref in zip(z["bf_track_args"], z["bf_track"]):
        got = np.array([gs.track_impedance(l, w, t)(x) for x in f])
        assert rel(got, ref) < 1e-13


def test_routed_board_is_the_rasterised_one():
    """routed_pair's fixture holds the board as raster.build_layer made it from its polygons: made again, the
    masks and labels are the same bit for bit and the widths, fills and areas to 1e-12 of their scale (with
    the same exact zeros)."""
    z, board = load("routed_pair")
    again = synth.routed_pair().to_arrays()
    for k, v in again.items():
        v, ref = np.asarray(v), z[f"board_{k}"]
        if v.dtype.kind == "f" and ref.dtype.kind == "f":
            scale = max(float(np.abs(ref).max(initial=0.0)), 1e-300)
            assert v.shape == ref.shape and np.array_equal(v == 0, ref == 0), k
            assert float(np.abs(v - ref).max(initial=0.0)) <= 1e-12 * scale, k
        else:
            assert np.array_equal(v, ref), k
