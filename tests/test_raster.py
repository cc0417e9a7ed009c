"""The exact-copper raster's arithmetic (groundtruth_gb300.raster) against GroundTruth's own outputs on seeded
polygons and arrays (tests/golden/raster_functions.npz, made by tests/golden/make_raster_golden.py), and the
copper area against the polygon's own area.  raster.py is an implementation of its own (scanline ramps, Green's
theorem over each cell's edge stretches, min-label pieces): masks, labels and indices must equal the
reference's bit for bit, float outputs agree to 1e-12 of their scale with the same exact zeros."""
from pathlib import Path

import numpy as np
import pytest

from groundtruth_gb300 import raster

Z = np.load(Path(__file__).resolve().parent / "golden" / "raster_functions.npz")


def close(got, ref, rel=1e-12) -> bool:
    """Floats of an independent implementation: within rel of the reference's scale, zero exactly where the
    reference's are (the masks built on them test > 0)."""
    got, ref = np.asarray(got, float), np.asarray(ref, float)
    scale = max(float(np.abs(ref).max()) if ref.size else 0.0, 1e-300)
    return got.shape == ref.shape and np.array_equal(got == 0, ref == 0) and float(np.abs(got - ref).max(initial=0.0)) <= rel * scale


def test_edges_put_the_copper_on_their_left():
    out, holes = np.array([[0, 0], [0, 4], [5, 4], [5, 0]], float), [np.array([[1, 1], [2, 1], [2, 2], [1, 2]], float)]
    pa, pb = raster.ring_edges(out, holes)
    area = 0.5 * np.sum(pa[:, 0] * pb[:, 1] - pb[:, 0] * pa[:, 1])       # shoelace over every oriented edge
    assert area == 20.0 - 1.0


def test_line_cover_and_cell_areas_match_reference():
    pa, pb = Z["pa"], Z["pb"]
    d, xl, yl, wi, wj = 0.35, 1.3, 1.1, 40, 42
    right = raster.line_cover(pa[:, 0], pa[:, 1], pb[:, 0], pb[:, 1], xl + d, d, wi, yl + d / 2, d, wj)
    top = raster.line_cover(pa[:, 1], pa[:, 0], pb[:, 1], pb[:, 0], yl + d, d, wj, xl + d / 2, d, wi)
    assert close(right, Z["right"]) and close(top, Z["top"])
    areas = raster.cell_areas(pa, pb, xl, yl, d, wi, wj, right)
    assert close(areas, Z["areas"])
    # the cells' areas add up to the polygon's (the grid covers it whole)
    poly = 0.5 * np.sum(pa[:, 0] * pb[:, 1] - pb[:, 0] * pa[:, 1])
    assert abs(areas.sum() - poly) < 1e-9 * poly


def test_strip_widths_adopt_and_series_factor_match_reference():
    args = [Z[f"sw_{k}"] for k in ("exists", "cross", "offset", "forced")]
    for w, o, exact in ((Z["sw_w0"], Z["sw_o0"], None), (Z["sw_w1"], Z["sw_o1"], Z["sw_exact"])):
        gw, go = raster.strip_widths(*args, 0.25, exact)
        assert close(gw, w) and close(go, o)
    steps = [(0, 1), (0, -1), (1, 0), (-1, 0)]
    assert close(raster.adopt(Z["ad_cov"], Z["ad_has"], steps), Z["ad_1"])
    assert close(raster.adopt(Z["ad_cov"], Z["ad_has"], steps, 3), Z["ad_3"])
    for ax in (0, 1):
        got = raster.series_factor(Z["sf_face"], list(Z["sf_samples"]), Z["sf_has"], ax)
        assert close(got, Z[f"sf_{ax}"])


def test_exact_widths_of_a_slanted_slot():
    """A plane with a slanted slot rasterised with exact widths: full strips away from it, strips whose border
    the slot partly covers narrower, every width in (0, 1]; the host stack models them."""
    from groundtruth_gb300 import stack as gs, synth
    d, n = 0.5e-3, 30
    h = d / 2
    outline = np.array([[-h, -h], [(n - 1) * d + h, -h], [(n - 1) * d + h, (n - 1) * d + h], [-h, (n - 1) * d + h]])
    slot = synth.rect_polygon(7.3e-3, 7.1e-3, 9e-3, 0.8e-3, 0.5)
    node, xb, yb, w = synth.raster_layer(n, n, d, outline, [slot], exact=True)
    wx, wy = w["wx"][xb], w["wy"][yb]
    assert np.all((wx > 0) & (wx <= 1)) and np.all((wy > 0) & (wy <= 1))
    narrow = lambda w: np.count_nonzero(w < 1 - 1e-9)      # noqa: E731  (a border's sum of partial intervals)
    assert 0 < narrow(wx) < len(wx) // 4 and narrow(wy) > 0
    layer = synth.Layer("GND", 0.0, 35e-6, node, xb, yb, w)
    pwr = synth._full_layer("PWR", -0.5e-3, 35e-6, n, n, d)
    b = synth.Board("exact", d, n, n, [layer, pwr], [synth.Pair(0, 1, 7.6e-8, 0.02)], [], [], np.array([1e8]))
    st, _ = gs.from_board(b, _device=False)
    assert st.dL is not None and np.count_nonzero(st.dL) == narrow(st.strip_width)


def _lines():
    ptr = Z["tr_ptr"]
    return [(Z["tr_pts"][a:b], float(w)) for a, b, w in zip(ptr[:-1], ptr[1:], Z["tr_width"])]


def test_track_walk_matches_reference():
    """raster.rasterise_tracks against the reference's _rasterise_lines on seeded layers (free cells, the net's
    own cells, other nets' cells) with polylines running off the grid, without and with pieces of copper: the
    claimed labels, seeded cells, forced strip widths, pieces and bridges, bit for bit."""
    lines = _lines()
    for case in ("plain", "pieces"):
        label = Z[f"tr_{case}_label0"].copy()
        nx, ny = label.shape
        seeded = np.zeros((nx, ny), bool)
        fx, fy = np.zeros((nx - 1, ny)), np.zeros((nx, ny - 1))
        part = Z[f"tr_{case}_part0"].copy() if case == "pieces" else None
        owners = list(Z["tr_owners"]) if case == "pieces" else None
        br = raster.rasterise_tracks(2, lines, 1.0, 2.0, 0.5, label, seeded, fx, fy, part, owners)
        assert np.array_equal(label, Z[f"tr_{case}_label"])
        assert np.array_equal(seeded, Z[f"tr_{case}_seeded"])
        assert np.array_equal(fx, Z[f"tr_{case}_fx"]) and np.array_equal(fy, Z[f"tr_{case}_fy"])
        assert np.array_equal(np.array(br, float).reshape(-1, 6), Z[f"tr_{case}_bridges"])
        if part is not None:
            assert np.array_equal(part, Z[f"tr_{case}_part"])


def test_a_straight_track_on_free_cells_claims_one_row():
    """A track along a row of free cells claims that row, forces its x strips to the track's width and needs
    no bridge; a foreign cell in its way is walked around (the L path through fewer foreign cells)."""
    label = -np.ones((12, 7), np.int64)
    seeded = np.zeros(label.shape, bool)
    fx, fy = np.zeros((11, 7)), np.zeros((12, 6))
    br = raster.rasterise_tracks(1, [(np.array([[1.0, 3.0], [9.0, 3.0]]), 0.3)], 0.0, 0.0, 1.0, label, seeded, fx, fy)
    assert br == [] and np.array_equal(np.flatnonzero(label[:, 3] == 1), np.arange(1, 10))
    assert (label == 1).sum() == 9 and np.all(fx[1:9, 3] == 0.3) and not fy.any()
    label = -np.ones((12, 7), np.int64)
    label[5, 3] = 0                                       # another net's cell on the centreline
    seeded[:] = False
    fx[:], fy[:] = 0, 0
    br = raster.rasterise_tracks(1, [(np.array([[1.0, 3.0], [9.0, 3.0]]), 0.3)], 0.0, 0.0, 1.0, label, seeded, fx, fy)
    assert label[5, 3] == 0 and br == []                  # the walk stepped around it
    assert (label == 1).sum() > 9 and fy.any()


def _copper_nets():
    nets = []
    for k in range(3):
        holes = [Z[f"cu_net{k}_hole{m}"] for m in range(4) if f"cu_net{k}_hole{m}" in Z.files]
        nets.append((Z[f"cu_net{k}_outline"], holes))
    return nets


def test_sub_grid_rasteriser_matches_reference():
    """raster.coarse_from_fine against the reference's _coarse_from_fine (s = 4) on a pour with holes, a slanted
    0.3 mm track and a pad: the cells' nets bit for bit, the border crossings, their offsets and the fill to 1e-12 (the
    sub-grid's point test, synth.copper_at, stood in for shapely's in the reference run)."""
    got = raster.coarse_from_fine(_copper_nets(), 0.4, 0.3, 0.5, 44, 46, 4)
    assert np.array_equal(got[0], Z["cu_label"])
    for g, key in zip(got[1:], ("cx", "cy", "fill", "ox", "oy")):
        assert close(g, Z[f"cu_{key}"]), key


def test_exact_copper_matches_reference():
    """raster.exact_copper against the reference's _exact_copper on the same nets and cells: strip widths, node
    areas and the narrow track's series factors, to 1e-12; the areas add up to the copper's."""
    nets = [raster.ring_edges(o, h) for o, h in _copper_nets()]
    got = raster.exact_copper(nets, Z["cu_label"], Z["cu_xb"], Z["cu_yb"], 0.4, 0.3, 0.5)
    for g, key in zip(got, ("ex_x", "ex_y", "area", "kx", "ky")):
        assert close(g, Z[f"cu_{key}"]), key
    assert (got[3] != 1).any()                                # the narrow track's series factors
    copper = sum(0.5 * np.sum(pa[:, 0] * pb[:, 1] - pb[:, 0] * pa[:, 1]) for pa, pb in nets)
    assert abs(got[2].sum() * 0.25 - copper) < 0.02 * copper  # copper of no node within reach is dropped


def _layer_nets():
    nets = {}
    for name in ("GND", "SIG", "VCC"):
        pieces = []
        for m in range(3):
            if f"ly_{name}_{m}_outline" not in Z.files:
                break
            holes = [Z[f"ly_{name}_{m}_hole{q}"] for q in range(4) if f"ly_{name}_{m}_hole{q}" in Z.files]
            pieces.append((Z[f"ly_{name}_{m}_outline"], holes))
        nets[name] = pieces
    return nets


@pytest.mark.parametrize("case, bbox, d, sub", [("s1", (0.3, 0.2, 21.0, 24.5), 0.5, 1),
                                                ("s4", (0.3, 0.2, 21.0, 24.5), 0.5, 4),
                                                ("s3", (-0.4, 0.9, 20.6, 22.0), 0.7, 3)])
def test_layer_raster_matches_reference(case, bbox, d, sub):
    """raster.build_layer against the reference's build_grid on a layer with a pour (holes), a slanted track, a
    supply of two separate pads, seeds (one on a far empty node, one for a net the layer lacks) and tracks: nodes,
    strips, labels and bridges bit for bit at sub = 1, 4 and 3, and at sub = 4 and 3 the fill, strip widths and
    offsets, node areas and resistance widths to 1e-12 (the reference run with the same point test, its heat points left out)."""
    seeds = {"GND": [(4.0, 12.0), (10.1, 9.6), (2.9, 2.7)], "VCC": [(18.0, 4.0), (30.0, 30.0)], "NC": [(1.0, 1.0)]}
    lines = {"SIG": [(np.array([[5.2, 14.3], [11.0, 16.1], [19.4, 20.2]]), 0.2)],
             "GND": [(np.array([[3.0, 3.0], [3.0, 6.5], [6.0, 6.5]]), 0.25)],
             "VCC": [(np.array([[2.8, 2.6], [17.9, 3.9]]), 0.3)]}
    g = raster.build_layer(_layer_nets(), bbox, d, seeds, lines, sub)
    for key in ("node", "xb", "yb", "label"):
        assert np.array_equal(getattr(g, key), Z[f"ly_{case}_{key}"]), key
    assert np.array_equal(np.array(g.bridges, float).reshape(-1, 6), Z[f"ly_{case}_bridges"])
    for key in ("fill", "wx", "wy", "ox", "oy", "area", "rx", "ry"):
        if sub == 1:
            assert getattr(g, key) is None
        else:
            assert close(getattr(g, key), Z[f"ly_{case}_{key}"]), key
    if sub > 1:
        assert set(g.widths()) == {"wx", "wy", "ox", "oy", "rx", "ry"}


def _circle(cx, cy, r, n=32):
    a = 2 * np.pi * np.arange(n) / n
    return np.stack([cx + r * np.cos(a), cy + r * np.sin(a)], 1)


def _pieces_of(g) -> int:
    """Connected pieces of a layer's copper (nodes joined by strips)."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import connected_components
    n = g.nx * g.ny
    idx = np.arange(n).reshape(g.nx, g.ny)
    a = np.concatenate([idx[:-1, :][g.xb], idx[:, :-1][g.yb]])
    b = np.concatenate([idx[1:, :][g.xb], idx[:, 1:][g.yb]])
    _, lab = connected_components(sp.coo_matrix((np.ones(len(a)), (a, b)), shape=(n, n)), directed=False)
    return len(set(lab[g.node.ravel()].tolist()))


PLANE = np.array([[0.0, 0.0], [20.0, 0.0], [20.0, 10.0], [0.0, 10.0]])


def test_antipad_webs_conduct_on_the_sub_grid():
    """The reference's test_raster.py:24-32: 0.36 mm antipads every 0.5 mm along x = 10 leave 0.14 mm webs; point
    sampling on a 0.5 mm grid loses every node on that line (two pieces), the sub-grid keeps one piece with the
    webs' cells partly filled."""
    holes = [_circle(10.0, 0.5 * k, 0.18) for k in range(1, 20)]
    plane = {"P": [(PLANE, holes)]}
    assert _pieces_of(raster.build_layer(plane, (0, 0, 20, 10), 0.5)) == 2
    g = raster.build_layer(plane, (0, 0, 20, 10), 0.5, sub=5)
    assert _pieces_of(g) == 1
    assert 0.2 < g.fill[20, 4] < 1.0 and g.fill[5, 5] == 1.0


def test_a_slot_narrower_than_the_pitch_still_cuts():
    """test_raster.py:35-37: a 0.3 mm slot across the plane on a 0.5 mm grid with the sub-grid: two pieces."""
    halves = [(np.array([[0.0, 0.0], [9.85, 0.0], [9.85, 10.0], [0.0, 10.0]]), []),
              (np.array([[10.15, 0.0], [20.0, 0.0], [20.0, 10.0], [10.15, 10.0]]), [])]
    assert _pieces_of(raster.build_layer({"P": halves}, (0, 0, 20, 10), 0.5, sub=5)) == 2


def test_capacitance_follows_copper_fill():
    """test_raster.py:40-56: a plane pair's capacitance counts the copper facing in each cell (the cells' sub-grid
    fill), not whole cells: perforated planes (96 holes of 0.3 mm radius) have the capacitance of their area,
    within 3 %."""
    from groundtruth_gb300 import stack as gs
    holes = [_circle(2 + 1.0 * i, 2 + 1.0 * j, 0.3) for i in range(16) for j in range(6)]

    def capacitance(h):
        g = raster.build_layer({"P": [(PLANE, h)]}, (0, 0, 20, 10), 0.25, sub=4)
        grid = gs.Grid(0.0, 0.0, 0.25, g.nx, g.ny, g.node, g.xb, g.yb, **g.widths(), fill=g.fill, area=g.area)
        layers = [gs.PlaneLayer(n, z, grid) for n, z in (("top", 0.2e-3), ("bot", 0.0))]
        st = gs.PlaneStack(layers, capacitance=[gs.PlanePair(0, 1, 8.854e-12 * 4.5 / 0.2e-3, 0.0)], _device=False)
        return st.top.cap[:, 4].sum()

    def area(poly):
        return 0.5 * abs(np.sum(poly[:, 0] * np.roll(poly[:, 1], -1) - np.roll(poly[:, 0], -1) * poly[:, 1]))
    expected = (area(PLANE) - sum(area(h) for h in holes)) / area(PLANE)
    assert abs(capacitance(holes) / capacitance([]) - expected) < 0.03


@pytest.mark.parametrize("case, bbox, d, sub", [("s1", (0.3, 0.2, 21.0, 24.5), 0.5, 1),
                                                ("s4", (0.3, 0.2, 21.0, 24.5), 0.5, 4)])
def test_grid_lookups_match_reference(case, bbox, d, sub):
    """stack.Grid's nearest_node (any net, one net, within a distance, a net the layer lacks), net_at and extent
    (peec.py:225-327) on the rasterised layer against the reference's Grid."""
    from groundtruth_gb300 import stack as gs
    seeds = {"GND": [(4.0, 12.0), (10.1, 9.6), (2.9, 2.7)], "VCC": [(18.0, 4.0), (30.0, 30.0)], "NC": [(1.0, 1.0)]}
    lines = {"SIG": [(np.array([[5.2, 14.3], [11.0, 16.1], [19.4, 20.2]]), 0.2)],
             "GND": [(np.array([[3.0, 3.0], [3.0, 6.5], [6.0, 6.5]]), 0.25)],
             "VCC": [(np.array([[2.8, 2.6], [17.9, 3.9]]), 0.3)]}
    r = raster.build_layer(_layer_nets(), bbox, d, seeds, lines, sub)
    g = gs.Grid(r.x0, r.y0, r.d, r.nx, r.ny, r.node, r.xb, r.yb, label=r.label, nets=r.nets)
    near = []
    for x, y in [(2.0, 2.0), (10.3, 9.1), (17.9, 4.1), (12.0, 17.6), (30.0, 5.0), (0.0, 24.0)]:
        for net, dist in ((None, None), ("VCC", None), ("SIG", 1.0), ("GND", 0.3), ("NC", None)):
            n = g.nearest_node(x, y, dist, net)
            near.append((-1, -1) if n is None else n)
    assert np.array_equal(np.array(near), Z[f"ly_{case}_near"])
    assert [g.net_at(n) if n[0] >= 0 else "" for n in near] == list(Z[f"ly_{case}_net_at"])
    assert np.allclose(g.extent, Z[f"ly_{case}_extent"], rtol=0, atol=1e-15)


def _box(x0, y0, x1, y1):
    return (np.array([[x0, y0], [x1, y0], [x1, y1], [x0, y1]]), [])


def test_pieces_group_copper_that_touches():
    """raster.pieces (peec.py:852-873): polygons within PIECE_TOL (5 um) of each other, or inside one another's
    copper, are one piece (transitively); a real gap keeps them apart."""
    a, b, c = _box(0, 0, 10, 4), _box(10 + 1e-7, 0, 20, 4), _box(20.003, 0, 30, 4)
    assert len(raster.pieces([a, b, c])) == 1                        # a-b touch, b-c 3 um apart
    assert len(raster.pieces([a, _box(10.02, 0, 20, 4)])) == 2      # 20 um: two pieces
    island = _box(3, 1, 4, 2)
    ring = (np.array([[0.0, 0.0], [8.0, 0.0], [8.0, 8.0], [0.0, 8.0]]), [np.array([[2.0, 2.0], [6.0, 2.0],
                                                                                   [6.0, 6.0], [2.0, 6.0]])])
    assert len(raster.pieces([ring, _box(3, 3, 4, 4)])) == 2       # an island in a hole, 1 mm off its edge
    assert len(raster.pieces([_box(0, 0, 8, 8), island])) == 1      # inside the copper
    assert raster.pieces([a]) == [a]


def _dc_drop(layer_nets, drive, sink, d=0.5, sub=4, bbox=(0, 0, 30, 12)):
    """The DC resistance between two points of a one-layer copper rasterised by build_layer (oracle solve)."""
    from test_oracle_golden import oracle_routes, oracle_stack
    from groundtruth_gb300 import stack as gs, synth
    g = raster.build_layer(layer_nets, bbox, d, sub=sub)
    grid = gs.Grid(0.0, 0.0, d, g.nx, g.ny, g.node, g.xb, g.yb, **g.widths(), fill=g.fill, area=g.area)
    ends = [(0, *grid.nearest_node(*p)) for p in (drive, sink)]
    board = synth.Board("rail", d * 1e-3, g.nx, g.ny, [synth.Layer("F", 0.0, 35e-6, g.node, g.xb, g.yb, g.widths(),
                                                                   g.fill, g.area, g.label)],
                        nets=[synth.Net(np.zeros((0, 8)), *ends)], freqs=np.array([0.0]), tol=1e-12)
    gs.from_board(board, _device=False)              # the host's checks (connectivity) first
    return oracle_routes(oracle_stack(board), board)[0].solve(0.0, tol=1e-12)["Z_loop"].real


@pytest.mark.parametrize("gap, joined", [(1e-7, True), (0.02, False)])
def test_copper_that_touches_is_one_piece_and_a_real_gap_is_not(gap, joined):
    """test_track_width.py:263-285 (TW-12): two 10 x 4 mm fills end to end, gap apart, fed at either end:
    1e-7 mm apart they conduct as one 20 mm fill (the DC drop within 0.5 %), 0.02 mm apart they are not
    connected."""
    from groundtruth_gb300.stack import SolverError
    fills = raster.pieces([_box(5.0, 4.0, 15.0, 8.0), _box(15.0 + gap, 4.0, 25.0, 8.0)])
    if not joined:
        with pytest.raises(SolverError, match="not connected"):
            _dc_drop({"PWR": fills}, (6.0, 6.0), (24.0, 6.0))
        return
    whole = _dc_drop({"PWR": [_box(5.0, 4.0, 25.0, 8.0)]}, (6.0, 6.0), (24.0, 6.0))
    assert _dc_drop({"PWR": fills}, (6.0, 6.0), (24.0, 6.0)) == pytest.approx(whole, rel=0.005)
