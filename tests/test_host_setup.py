"""The host-side setup (topology, dense layout, spectra, Schur structure) against the oracle, through the
numpy model of the device algorithm (tests/host_model.py).  CPU only."""
import numpy as np
import pytest
import scipy.sparse as sp

from groundtruth_gb300 import stack as gs
from oracle import peec_oracle as po
from test_oracle_golden import load, oracle_stack
from host_model import DenseModel, Multifrontal

CASES = ["small_pair", "small_stack3", "plain_plane"]


@pytest.fixture(scope="module", params=CASES)
def case(request):
    z, board = load(request.param)
    st, routes = gs.from_board(board, _device=False)
    ost = oracle_stack(board)
    return request.param, z, board, st, routes, ost


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_topology_matches_reference(case):
    name, z, board, st, routes, ost = case
    for k in ("xa", "ya", "nid", "keep", "a_nodes", "b_nodes", "full_label", "cond_label"):
        assert np.array_equal(getattr(st.top, k), z[k]), k
    assert np.array_equal(st.top.cap, z["cap"])
    assert st.nb == int(z["nb"])


def test_dense_matvec_matches_oracle(case):
    name, z, board, st, routes, ost = case
    m = DenseModel(st)
    f = float(z["op_f"])
    op = ost.operator(f)
    w, zs, zcap, zbr, tab = st._freq_tables(f)
    x = z["prod_x"]
    got = m.to_compact(m.matvec(m.to_dense(x), w, zs, zcap, zbr))
    assert rel(got, z["prod_matvec"]) < 1e-12
    I = z["prod_I"]
    v = np.zeros(m.D.n, complex)
    v[m.D.compact_to_dense[: st.ns]] = I
    lp = np.concatenate([m.lp(m.seg(v, "X"), "x")[tuple(st.xa.T)], m.lp(m.seg(v, "Y"), "y")[tuple(st.ya.T)]])
    assert rel(lp, z["prod_Lp"]) < 1e-12


def test_schur_assembly_and_factor_match_oracle(case):
    name, z, board, st, routes, ost = case
    f = float(z["op_f"])
    op = ost.operator(f)
    w, zs, zcap, zbr, tab = st._freq_tables(f)
    svals = st.sterm @ tab
    sym = st.sym
    n = sym.n
    Sl = sp.coo_matrix((svals, (sym.s_row, sym.s_col)), shape=(n, n)).toarray()
    Sfull = np.tril(Sl) + np.tril(Sl, -1).T
    # oracle S in reference kept order -> factor order
    node_dense = np.flatnonzero(st.top.node.ravel())
    fac = sym.perm[node_dense[st.top.keep]]
    So = np.zeros((n, n), complex)
    Sd = op["S"].toarray()
    So[np.ix_(fac, fac)] = Sd
    assert np.abs(Sfull - So).max() <= 1e-12 * np.abs(So).max()
    mf = Multifrontal(st, svals)
    b = np.random.default_rng(0).standard_normal(n) + 1j * np.random.default_rng(1).standard_normal(n)
    y = mf.solve(b)
    assert rel(Sfull @ y, b) < 1e-10


def test_dense_precond_matches_oracle(case):
    name, z, board, st, routes, ost = case
    m = DenseModel(st)
    f = float(z["op_f"])
    w, zs, zcap, zbr, tab = st._freq_tables(f)
    mf = Multifrontal(st, st.sterm @ tab)
    got = m.to_compact(m.precond(m.to_dense(z["prod_x"]), tab, mf))
    assert rel(got, z["prod_precond"]) < 1e-9


def test_excitation_matches_reference(case):
    name, z, board, st, routes, ost = case
    for k, r in enumerate(routes):
        assert rel(r.psi, z[f"psi{k}"]) < 1e-13
        assert r.L_trace == pytest.approx(float(z[f"Ltrace{k}"]), rel=1e-13)


@pytest.mark.parametrize("name", ["small_pair", "necked_pair", "faces_stack3_diag", "faces_stack3_sheet", "necked_faces"])
def test_schur_values_and_impedances_match_reference(name):
    """The per-frequency admittance table through the S-term map gives the reference's own Schur complement
    (narrow strips' own blocks, split layers' face blocks included), and the table's impedances its R_strip and
    face coupling Z12."""
    z, board = load(name)
    st, routes = gs.from_board(board, _device=False)
    for k in ("xa", "ya", "keep", "a_nodes", "b_nodes"):
        assert np.array_equal(getattr(st.top, k), z[k]), k
    f = float(z["op_f"])
    w, zs, zcap, zbr, tab = st._freq_tables(f)
    sym = st.sym
    ij = z["op_S_ij"]
    S_ref = sp.coo_matrix((z["op_S"], (ij[0], ij[1])), shape=(sym.n, sym.n)).tocsr()
    fac = sym.perm[np.flatnonzero(st.top.node.ravel())[st.top.keep]]
    P = sp.coo_matrix((np.ones(sym.n), (fac, np.arange(sym.n))), shape=(sym.n, sym.n)).tocsr()
    ref = np.asarray((P @ S_ref @ P.T).tocsr()[sym.s_row, sym.s_col]).ravel()
    # the impedances are this build's own FP64 arithmetic: rounding differences of 1e-16 grow through the face
    # blocks' inverses, so the values agree to 1e-12 of the largest
    assert np.abs(st.sterm @ tab - ref).max() <= 1e-12 * np.abs(ref).max()
    R = zs[: st.n_sheets][np.concatenate([st.xa[:, 0], st.ya[:, 0]])] / st.r_width
    assert rel(R, z["op_R"]) < 1e-14
    if "op_Z12" in z.files:
        Z12 = zs[st.n_sheets:][st.sheet_of_strip(st.tw_b) - st.N] / st.r_width[st.tw_b]
        assert rel(Z12, z["op_Z12"]) < 1e-14


@pytest.mark.parametrize("name", ["necked_pair_scaled", "faces_stack3_sheet_scaled"])
def test_resistance_scale_tables(name):
    """set_resistance_scale on the host side: the scaled strips' own D^-1 blocks through the S-term map give
    the (pinned) oracle's Schur complement, the scaled impedances the reference's R_strip and branch z."""
    z, board = load(name)
    st, routes = gs.from_board(board, _device=False)
    st.set_resistance_scale(z["r_scale"], z["branch_scale"])
    ost = oracle_stack(board)
    ost.set_resistance_scale(z["r_scale"], z["branch_scale"])
    f = float(z["op_f"])
    op = ost.operator(f)
    w, zs, zcap, zbr, tab = st._freq_tables(f)
    sym = st.sym
    fac = sym.perm[np.flatnonzero(st.top.node.ravel())[st.top.keep]]
    P = sp.coo_matrix((np.ones(sym.n), (fac, np.arange(sym.n))), shape=(sym.n, sym.n)).tocsr()
    ref = np.asarray((P @ op["S"].tocsr() @ P.T).tocsr()[sym.s_row, sym.s_col]).ravel()
    assert np.abs(st.sterm @ tab - ref).max() <= 1e-13 * np.abs(ref).max()
    assert rel(zbr, z["op_z"][st.ncap:]) < 1e-14
    nr = st.narrow_rows
    sc = z["r_scale"]
    assert np.count_nonzero(nr["rre"]) == np.count_nonzero((sc != 1.0))


@pytest.mark.parametrize("name", ["necked_pair_fields", "routed_pair_fields"])
def test_current_density_maps_match_reference(name):
    """Solution.node_field per cell width and per copper width (peec.py:1151-1203, Grid.copper_area 257-312) on
    the reference's own solution of a board with narrow strips, and of one rasterised from polygons whose nodes
    carry measured copper areas (the area spread over each node's 3 x 3 neighbourhood of its net)."""
    z, board = load(name)
    st, routes = gs.from_board(board, _device=False)
    x = z["x"]
    V = np.zeros(st.n_nodes, complex)
    V[st.keep] = x[st.nb:]
    sol = routes[0].solution(float(z["f"]), x[: st.nb], V, 0)
    for k in range(st.N):
        for copper in (False, True):
            kx, ky = sol.node_field(k, board.d * 1e3, copper=copper)
            assert rel(kx, z[f"kx{k}_{int(copper)}"]) < 1e-12 and rel(ky, z[f"ky{k}_{int(copper)}"]) < 1e-12
            vx, vy = sol.sheet_vectors(k, board.d * 1e3, copper=copper)
            assert rel(vx, z[f"vx{k}_{int(copper)}"]) < 1e-12 and rel(vy, z[f"vy{k}_{int(copper)}"]) < 1e-12
    # the dominant phase (peec.py:1210-1226) and the layers' current shares (1235-1247)
    assert sol.dominant_phase() == pytest.approx(float(z["phase"]), abs=1e-12)
    assert np.allclose(sol.layer_share(), z["share"], rtol=1e-12, atol=0)
    masks = [(np.ones(sol.I_x[k].shape, bool), np.zeros(sol.I_y[k].shape, bool)) for k in range(st.N)]
    assert np.allclose(sol.layer_share(masks), z["share_masked"], rtol=1e-12, atol=0)


@pytest.mark.parametrize("name", ["necked_pair", "faces_stack3_diag", "faces_stack3_sheet", "necked_faces",
                                  "necked_pair_scaled", "faces_stack3_sheet_scaled", "routed_pair"])
def test_corrections_and_face_sheets_through_the_device_model(name):
    """The arrays uploaded for strips narrower than the pitch, face sheets and resistance factors (the correction
    rows, the positions' own D^-1 blocks, the sheets' node layers) give, through the numpy model of the device
    algorithm, the reference's own system product (<=1e-12) and preconditioner (<=1e-9)."""
    z, board = load(name)
    st, routes = gs.from_board(board, _device=False)
    if "r_scale" in z.files:
        st.set_resistance_scale(z["r_scale"], z["branch_scale"])
    m = DenseModel(st)
    f = float(z["op_f"])
    w, zs, zcap, zbr, tab = st._freq_tables(f)
    x = m.to_dense(z["prod_x"])
    got = m.to_compact(m.matvec(x, w, zs, zcap, zbr))
    assert rel(got, z["prod_matvec"]) < 1e-12
    rows = np.flatnonzero(np.isin(m.D.compact_to_dense, st.narrow_rows["pos"]))     # the corrected rows alone
    assert len(rows) and rel(got[rows], z["prod_matvec"][rows]) < 1e-12
    mf = Multifrontal(st, st.sterm @ tab)
    pc = m.to_compact(m.precond(x, tab, mf))
    assert rel(pc, z["prod_precond"]) < 1e-9
    if st.ncap and np.any(st.top.cap_share != 1.0):      # partly covered cells: their rows alone
        cap = np.arange(st.ns, st.ns + st.ncap)
        assert rel(got[cap], z["prod_matvec"][cap]) < 1e-12 and rel(pc[cap], z["prod_precond"][cap]) < 1e-9


def test_derived_stack_through_the_device_model():
    """A derived stack (a what-if edit's branches on the base's factorisation, PlaneStack.with_branches): its
    system product and its preconditioner, the base's factor with the low-rank update for the added branches,
    through the numpy model equal the reference's own derived stack's (small_pair_derived.npz)."""
    from host_model import LowRank
    from test_derived_stacks import extra_of
    z, board = load("small_pair_derived")
    st, _ = gs.from_board(board, _device=False)
    dst = st.with_branches([gs.Branch(b.a, b.b, b.z, f"x{n}", b.kind, b.radius)
                            for n, b in enumerate(extra_of(z))])
    assert dst._base is st and dst.n_lowrank > 0
    m = DenseModel(dst)
    w, zs, zcap, zbr, tab = dst._freq_tables(float(board.freqs[0]))
    x = m.to_dense(z["prod_x"])
    assert rel(m.to_compact(m.matvec(x, w, zs, zcap, zbr)), z["prod_matvec"]) < 1e-12
    base = Multifrontal(dst, dst.sterm @ tab[: st.n_table])
    assert rel(m.to_compact(m.precond(x, tab, LowRank(m, base, zbr))), z["prod_precond"]) < 1e-9
    assert rel(m.to_compact(m.precond(x, tab, base)), z["prod_precond"]) > 1e-3     # the update matters


def test_capacitance_shares_reach_the_device_cells():
    """native.cap_fill_cells (the descriptor's cap_fill) puts each capacitance's facing share at its own cell of
    the C segment, as the numpy device model applies it; None for whole cells."""
    from groundtruth_gb300 import native
    z, board = load("routed_pair")
    st, _ = gs.from_board(board, _device=False)
    cells = native.cap_fill_cells(st)
    assert cells is not None and np.array_equal(cells, DenseModel(st).share.ravel())
    st0, _ = gs.from_board(load("small_pair")[1], _device=False)
    assert native.cap_fill_cells(st0) is None
