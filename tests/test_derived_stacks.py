"""Derived stacks (PlaneStack.with_branches: a what-if edit's added branches on a base's factorisation, updated
by the Woodbury identity; peec.py:1871-1923, 2354-2377) on the CPU: the oracle's restatement against the
reference's own derived-stack outputs (tests/golden/small_pair_derived.npz), the Woodbury update against a
fresh factorisation of the whole stack, and the host side of the GPU build's derived stacks (branch filtering,
unknown numbering, warm-start mapping) without a device."""
import numpy as np
import pytest

from groundtruth_gb300 import stack as gs, synth
from oracle import peec_oracle as po
from test_oracle_golden import load, oracle_routes, oracle_stack


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


def extra_of(z):
    """The edit's branches as synth.BranchSpec rows (a, b, R, L, C, is_via, radius)."""
    out = []
    for r in z["extra"]:
        a, b = tuple(int(v) for v in r[0:3]), tuple(int(v) for v in r[3:6])
        out.append(synth.BranchSpec(a, b, float(r[6]), float(r[7]), float(r[8]), "via" if r[9] else "part",
                                    float(r[10])))
    return out


@pytest.fixture(scope="module")
def derived():
    z, board = load("small_pair_derived")
    extra = extra_of(z)
    ost = oracle_stack(board)
    odst = ost.with_branches([po.OBranch(b.a, b.b, b.R, b.L, b.C, b.kind, b.radius) for b in extra])
    return z, board, extra, ost, odst


def test_fixture_edit_is_the_seeded_one(derived):
    z, board, extra, ost, odst = derived
    again = synth.what_if_branches(board, seed=11)
    assert [(b.a, b.b, b.kind) for b in again] == [(b.a, b.b, b.kind) for b in extra]


def test_oracle_derived_stack_is_derived(derived):
    z, board, extra, ost, odst = derived
    assert odst._base is ost
    assert odst.nb == int(z["nb"]) and odst.nbr == int(z["nbr"])
    assert np.array_equal(odst.keep, ost.keep)


def test_oracle_derived_products_match_reference(derived):
    z, board, extra, ost, odst = derived
    op = odst.operator(float(board.freqs[0]))
    assert rel(odst.matvec(op, z["prod_x"]), z["prod_matvec"]) < 1e-12
    assert rel(odst.precond(op, z["prod_x"]), z["prod_precond"]) < 1e-10


def test_woodbury_equals_fresh_factorisation(derived):
    """The update is exact: the derived stack's preconditioner is the whole stack's own."""
    z, board, extra, ost, odst = derived
    full = po.OracleStack(ost.layers, ost.d, ost.branches + list(odst.branches[ost.nbr:]), ost.pairs, ost.sigma,
                          ost.precond_mode)
    assert full._base is None and full.nb == odst.nb
    for f in board.freqs:
        a, b = odst.operator(float(f)), full.operator(float(f))
        assert rel(odst.precond(a, z["prod_x"]), full.precond(b, z["prod_x"])) < 1e-10


def test_oracle_derived_solves_match_reference(derived):
    z, board, extra, ost, odst = derived
    routes = oracle_routes(odst, board)
    for k, r in enumerate(routes):
        assert rel(r.psi, z[f"psi{k}"]) < 1e-12
        q = 1
        ref = r.solve(float(board.freqs[q]), tol=board.tol)
        assert abs(ref["Z_loop"] - z[f"Z{k}_{q}"]) <= 1e-8 * abs(z[f"Z{k}_{q}"])
        assert rel(ref["x"][: odst.nb], z[f"x{k}_{q}"][: odst.nb]) < 1e-7


def test_oracle_map_state(derived):
    z, board, extra, ost, odst = derived
    x = np.arange(ost.nb + int(ost.keep.sum())).astype(complex)
    y = odst.map_state(x, ost)
    assert len(y) == odst.nb + int(odst.keep.sum())
    assert np.array_equal(y[: ost.nb], x[: ost.nb]) and not y[ost.nb: odst.nb].any()
    assert np.array_equal(y[odst.nb:], x[ost.nb:])


# ---------------------------------------------------------------------------------------- host side of the build
def host_stack(board):
    return gs.from_board(board, _device=False)[0]


def branches_of(extra):
    return [gs.Branch(b.a, b.b, b.z, f"x{n}", b.kind, b.radius) for n, b in enumerate(extra)]


def test_with_branches_numbering(derived):
    z, board, extra, ost, odst = derived
    st = host_stack(board)
    dst = st.with_branches(branches_of(extra))
    assert dst._base is st and dst.n_lowrank == len(extra)
    assert dst.nb == int(z["nb"]) and dst.nbr == int(z["nbr"])
    assert np.array_equal(dst.keep, st.keep) and dst.sym is st.sym and dst.spectrum is st.spectrum
    # the dense layout gains the branches; the strips, caps and nodes keep their places
    assert dst.dense.off_b == st.dense.off_b and dst.dense.n >= st.dense.n
    c2d_base, c2d = st.dense.compact_to_dense, dst.dense.compact_to_dense
    assert np.array_equal(c2d[: st.nb], c2d_base[: st.nb])
    assert np.array_equal(c2d[dst.nb:] - dst.dense.off_v, c2d_base[st.nb:] - st.dense.off_v)
    # the admittance table grows by the added branches; the S-term map stays the base's
    assert dst.n_table == st.n_table + len(extra) and dst.sterm is st.sterm
    w, zs, zcap, zbr, tab = dst._freq_tables(1e8)
    assert np.allclose(tab[dst.tab_br0 + st.nbr:], [1.0 / b.z(1e8) for b in extra])


def test_with_branches_filters_and_chains(derived):
    z, board, extra, ost, odst = derived
    st = host_stack(board)
    assert st.with_branches([]) is st
    off = gs.Branch((0, 0, 0), (0, 0, 0), lambda f: 1.0)                 # both ends on one node
    outside = gs.Branch((0, 1, 1), (1, board.nx + 3, 1), lambda f: 1.0)  # an end off the grid
    assert st.with_branches([off, outside]) is st
    b = branches_of(extra)
    d1 = st.with_branches(b[:1])
    d2 = d1.with_branches(b[1:])
    assert d2._base is st and d2.n_lowrank == len(extra)              # derived from the first base
    x1 = np.arange(d1.nb + int(d1.keep.sum())).astype(complex)
    y = d2.map_state(x1, d1)
    assert len(y) == d2.nb + int(d2.keep.sum()) and not y[d1.nb: d2.nb].any()
    assert d2.map_state(x1, st) is None                                # not st's vector length


def test_with_branches_joining_copper_makes_a_stack():
    """Two sheets with no plane pair and no branch are separate pieces: a via between them changes the
    reference nodes, so the result is a stack of its own (peec.py:1880-1882)."""
    b = synth.small_pair()
    b.pairs, b.branches = [], []
    st = host_stack(b)
    via = gs.Branch((0, 20, 3), (1, 20, 3), lambda f: 1e-3 + 0j, "v", "via")
    assert st.full_label[st.node_id((0, 20, 3))] != st.full_label[st.node_id((1, 20, 3))]
    new = st.with_branches([via])
    assert new is not st and new._base is None and new.nbr == 1
    assert int(new.keep.sum()) == int(st.keep.sum()) + 1


def test_route_on_derived_reuses_strip_coupling(derived):
    z, board, extra, ost, odst = derived
    st, routes = gs.from_board(board, _device=False)
    dst = st.with_branches(branches_of(extra))
    r = routes[0].on(dst)
    assert r.strip_psi is routes[0].strip_psi
    assert len(r.psi) == dst.nb and rel(r.psi, z["psi0"]) < 1e-12


class _OracleBacked:
    """A host-only PlaneStack whose solves run on the oracle (FP64 CPU): the what-if composition's host
    arithmetic tested without a device."""

    def __init__(self, st, ost):
        self.st, self.ost = st, ost

    def solve_batch(self, freqs, rhs_tops, Js, tol=1e-5, guesses=None, failed=None, **kw):
        out = []
        for f, top, J in zip(freqs, rhs_tops, Js):
            Ib, V, its, x = self.ost.solve(f, np.asarray(top, complex), np.asarray(J, float), tol=tol)
            rhs = self.st.rhs_vector(top, J)
            res = np.linalg.norm(rhs - self.ost.matvec(self.ost.operator(f), x)) / np.linalg.norm(rhs)
            out.append((Ib, V, its, x, res))
        return out


def test_bordered_edit_composition_on_cpu(derived):
    """whatif.WhatIf's bordered way (base solves of the new branches' injections, k x k solve per column)
    with the oracle as the solver: loop impedance, moment, currents and the residual bound against the oracle's
    solve of the whole edited board."""
    from groundtruth_gb300 import whatif
    z, board, extra, ost, odst = derived
    st, routes = gs.from_board(board, _device=False)
    backed = _OracleBacked(st, ost)
    st.factorise = lambda *a, **k: None
    st.solve_batch = backed.solve_batch
    wi = whatif.WhatIf(st, routes, board.freqs[:2], tol=1e-9, method="bordered")
    wi.baseline()
    res = wi.evaluate(branches_of(extra), [0, 1], [float(board.freqs[1])])
    assert res.parts["border_columns"] == len(extra) and res.parts["cold_redo"] == 0
    oroutes = oracle_routes(odst, board)
    f = float(board.freqs[1])
    for k in (0, 1):
        col = res.solutions[(k, f)]
        ref = oroutes[k].solve(f, tol=1e-12)
        assert abs(col.Z_loop - ref["Z_loop"]) <= 1e-7 * abs(ref["Z_loop"])
        assert np.linalg.norm(col.m - ref["m"]) <= 1e-6 * np.linalg.norm(ref["m"])
        assert col.residual <= 1e-9
        sol = col.solution()
        x = sol.state_for(st.with_branches(branches_of(extra)))
        assert rel(x[: odst.nb], ref["x"][: odst.nb]) < 1e-6


def test_moved_part_composition_on_cpu(derived):
    """A moved decoupling part (removed at its place, added at another) through the bordered composition equals
    the oracle's solve of the board with the part moved."""
    from groundtruth_gb300 import whatif
    z, board, extra, ost, odst = derived
    st, routes = gs.from_board(board, _device=False)
    backed = _OracleBacked(st, ost)
    st.factorise = lambda *a, **k: None
    st.solve_batch = backed.solve_batch
    wi = whatif.WhatIf(st, routes, board.freqs[1:2], tol=1e-9)
    wi.baseline()
    decap = board.branches[0]
    moved = synth.BranchSpec((0, 30, 10), (1, 30, 10), decap.R, decap.L, decap.C, decap.kind, decap.radius)
    res = wi.evaluate(branches_of([moved]), [0], [float(board.freqs[1])], remove=[0])
    whole = synth.Board.from_arrays(board.to_arrays())
    whole.branches = [moved] + list(board.branches[1:])
    wst = oracle_stack(whole)
    ref = oracle_routes(wst, whole)[0].solve(float(board.freqs[1]), tol=1e-12)
    col = res.solutions[(0, float(board.freqs[1]))]
    assert abs(col.Z_loop - ref["Z_loop"]) <= 1e-7 * abs(ref["Z_loop"])
    assert np.linalg.norm(col.m - ref["m"]) <= 1e-6 * np.linalg.norm(ref["m"])


def test_with_branches_on_a_face_sheet_stack():
    """A derived stack of a stack with split layers keeps its sheets, twins and corrections."""
    z, board = load("faces_stack3_sheet")
    st = host_stack(board)
    more = synth.what_if_branches(board, seed=5, n_via=2, n_part=1)
    dst = st.with_branches(branches_of(more))
    assert dst._base is st and dst.n_sheets == st.n_sheets == 4
    assert np.array_equal(dst.tw_a, st.tw_a) and np.array_equal(dst.top.sheet_layer, st.top.sheet_layer)
    assert dst.nb == st.nb + len(more) and np.array_equal(dst.keep, st.keep)


def test_solves_split_into_what_fits_the_device(monkeypatch):
    """The memory gate: a batch whose workspace does not fit the free device memory is solved in parts, a
    column that does not fit at all raises MemoryError."""
    from groundtruth_gb300 import native
    st = host_stack(synth.small_pair())
    st.handle = object()
    per, fixed = 10, 5

    def fake_memory(geom, n, restart=50, precision="mixed", outer_k=8):
        return {"need": fixed + per * n, "held": 0, "free": free[0], "total": 10 ** 6}
    monkeypatch.setattr(native, "memory", fake_memory)
    free = [10 ** 6]
    assert st.columns_that_fit(40) == 40
    free[0] = (fixed + per * 12) / st.MEMORY_HEADROOM
    assert st.columns_that_fit(40) == 12
    free[0] = 1
    with pytest.raises(MemoryError):
        st.columns_that_fit(40)


def test_borrowed_columns_that_miss_get_their_own_factorisation(monkeypatch):
    """A column whose borrowed preconditioner does not reach the tolerance is factorised at its own frequency
    and solved on from where it got (peec.py:2584-2595); host logic with the device calls faked."""
    from groundtruth_gb300 import native
    st = host_stack(synth.small_pair())
    st.handle = object()
    freqs = [1e8, 1.1e8]

    class Obj:
        def __init__(self, keys, factor_of):
            self.keys, self.factor_of = keys, factor_of
    calls = []

    def fake_factorise(fs, together=False, borrow=False):
        keys = [gs.freq_key(f) for f in fs]
        obj = Obj(keys, np.array([0] * len(keys)) if borrow and len(keys) > 1 else None)
        return [(obj, n) for n in range(len(keys))]

    def fake_solve(geom, ops, rhs, tol, x0=None, **kw):
        obj = ops[0][0]
        calls.append((obj.factor_of is not None, x0 is not None))
        n = rhs.shape[0]
        x = np.ones_like(rhs) if x0 is None else x0 + 1
        res = np.array([1e-3 if obj.factor_of is not None and k == 1 else 1e-9 for k in range(n)])
        return x, np.full(n, 10, np.int32), res, res <= tol
    monkeypatch.setattr(st, "factorise", fake_factorise)
    monkeypatch.setattr(st, "columns_that_fit", lambda n, *a: n)
    monkeypatch.setattr(st, "_warm_start", lambda ops, rhs, guesses: np.stack([g[0] for g in guesses]))
    monkeypatch.setattr(native, "solve", fake_solve)
    J = np.zeros(st.n_nodes)
    out = st.solve_batch(freqs, [np.zeros(st.nb, complex)] * 2, [J, J], tol=1e-6, borrow=True)
    assert calls == [(True, False), (False, True)]          # the miss re-solved with its own, from its x
    assert out[1][2] == 20 and out[1][4] <= 1e-6


def test_factorisations_are_admitted_against_free_memory(monkeypatch):
    """The memory gate for factorisations: cached ones and the solve workspace are dropped when new ones would
    not fit, MemoryError when they still do not."""
    from groundtruth_gb300 import native
    st = host_stack(synth.small_pair())
    trims = []

    class Handle:
        def trim(self):
            trims.append(1)
    st.handle = Handle()
    one = st.factorisation_bytes(1)
    assert one > st.sym.panel_total * 48 and st.factorisation_bytes(4) == 4 * one
    free = [10 * one]
    monkeypatch.setattr(native, "memory", lambda g, n, *a, **k: {"need": 0, "held": 0, "free": free[0], "total": 0})
    st._ops["k"] = ("cached", 0)
    st._admit(4)
    assert "k" in st._ops                           # fits: the cache stays
    free[0] = 2 * one
    with pytest.raises(MemoryError):
        st._admit(4)
    assert not st._ops and trims                    # dropped before giving up


@pytest.mark.parametrize("name", ["small_pair", "capacitance_only", "faces_stack3", "six_sheet"])
def test_added_branches_number_like_a_whole_topology(name):
    """layout.add_branches (a derived stack's numbering without redoing the grid's work) gives exactly what
    layout.topology gives for the whole branch list: incidence ends, conductor components (merged and numbered
    by their lowest node, as connected_components numbers them), copper components and reference nodes.
    capacitance_only: the plane pair without its branches, its planes joined by capacitance alone, so a new via
    merges two conductor components."""
    from groundtruth_gb300 import layout
    board = synth.small_pair() if name in ("small_pair", "capacitance_only") else getattr(synth, name)()
    if name == "capacitance_only":
        board.branches = []
    st = host_stack(board)
    t0 = st.top
    coords = np.argwhere(t0.node)                        # node id -> (layer, i, j)
    rng = np.random.default_rng(7)
    merged = False
    for trial in range(6):
        ab = []
        while len(ab) < 1 + trial % 4:
            a, b = rng.integers(0, t0.n_nodes, 2)
            if a != b and t0.full_label[a] == t0.full_label[b]:
                ab.append((a, b))
        ab = np.array(ab)
        got = layout.add_branches(t0, ab)
        whole, kept = layout.topology([l.grid.node for l in st.layers], [l.grid.xb for l in st.layers],
                                      [l.grid.yb for l in st.layers], st.d,
                                      [(p.upper, p.lower, p.c_per_area, p.tan_delta) for p in st.pairs],
                                      [(br.a, br.b) for br in st.branches]
                                      + [(tuple(coords[a]), tuple(coords[b])) for a, b in ab], st.twin_parent)
        assert len(kept) == st.nbr + len(ab)
        for k in ("branch_ab", "a_nodes", "b_nodes", "cond_label", "full_label", "keep", "nid", "xa", "ya", "cap"):
            assert np.array_equal(getattr(got, k), getattr(whole, k)), (k, trial)
        merged |= got.cond_label.max() < t0.cond_label.max()
    assert merged == (name == "capacitance_only")
    other = np.flatnonzero(t0.full_label != t0.full_label[0])
    if len(other):                                       # a branch between two pieces of copper: a stack of its own
        with pytest.raises(ValueError):
            layout.add_branches(t0, [(0, other[0])])
