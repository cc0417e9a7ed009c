"""Seeded synthetic boards for the solver's workloads.

A board here is what GroundTruth hands its PEEC solver after rasterising copper (peec.build_grid with
sub=1, src/groundtruth/solver/peec.py:329-449): per plane layer a node mask and x/y strip masks on one
shared grid, the layers' heights and copper thickness, plane-pair capacitances, lumped branches, and per
net the known signal path as straight filaments with its driver / receiver return nodes.

Rasterisation follows the sub=1 rules of peec.py:385-393 and 432-435: a node is copper when its point lies
strictly inside the copper (shapely.contains_xy: a point on an edge is outside), an x strip exists when
both end nodes and the midpoint half a pitch to the right are copper of the net, a y strip likewise with the
midpoint half a pitch up.  Copper is a board outline minus cut-outs, both polygons.

Workloads (metres unless named otherwise):

* ``plain_plane``   one solid plane 96 x 96 at 0.5 mm, a 0.2 mm trace 0.2 mm above it from cell (10, 48)
                    to (86, 48), 100 MHz (the reference's CPU-runnable case).
* ``slotted_pair``  Sig/GND/PWR/Sig, gaps 0.2/1.0/0.2 mm, 256 x 256 at 0.25 mm, a seeded 1 mm slot across
                    60 % of the GND plane, 8 Manhattan random-walk nets crossing it, 32 log-spaced
                    frequencies 1 MHz - 1 GHz (8 x 32 = 256 solves).
* ``small_*``       reduced boards of the same kinds for golden fixtures and fast tests.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

EPS0 = 8.8541878128e-12
SIGMA_CU = 5.8e7
MU0 = 4e-7 * math.pi


# ------------------------------------------------------------------------------------------ geometry
def polygon_contains(px: np.ndarray, py: np.ndarray, poly: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(strictly inside, on the boundary) for points against a simple polygon (k, 2), crossing-number rule
    with an exact on-edge test, FP64, vectorised over the points."""
    px = np.asarray(px, float)
    py = np.asarray(py, float)
    inside = np.zeros(px.shape, bool)
    on_edge = np.zeros(px.shape, bool)
    n = len(poly)
    for e in range(n):
        x1, y1 = poly[e]
        x2, y2 = poly[(e + 1) % n]
        cross = (x2 - x1) * (py - y1) - (y2 - y1) * (px - x1)
        within = ((np.minimum(x1, x2) <= px) & (px <= np.maximum(x1, x2))
                  & (np.minimum(y1, y2) <= py) & (py <= np.maximum(y1, y2)))
        on_edge |= (cross == 0.0) & within
        straddle = (y1 > py) != (y2 > py)
        with np.errstate(divide="ignore", invalid="ignore"):
            xint = x1 + (py - y1) * (x2 - x1) / (y2 - y1)
        inside ^= straddle & (px < xint)
    return inside & ~on_edge, on_edge


def copper_at(px, py, outline: np.ndarray, cutouts: list) -> np.ndarray:
    """Points strictly inside the copper = outline minus the closed cut-outs (contains_xy semantics)."""
    inside, _ = polygon_contains(px, py, outline)
    for c in cutouts:
        cin, con = polygon_contains(px, py, c)
        inside &= ~(cin | con)
    return inside


def raster_layer(nx: int, ny: int, d: float, outline: np.ndarray, cutouts: list, exact: bool = False):
    """(node, xb, yb) masks for one layer's copper by the sub=1 rules (node at (i d, j d), coordinates in
    the same unit as d); exact=True adds the strips' widths: the share of each strip's cell border that the
    copper covers (raster.line_cover along the borders, raster.strip_widths), as (node, xb, yb, widths)."""
    xs = np.arange(nx) * d
    ys = np.arange(ny) * d
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    node = copper_at(X, Y, outline, cutouts)
    mx = copper_at(X[:-1, :] + d / 2, Y[:-1, :], outline, cutouts)
    my = copper_at(X[:, :-1], Y[:, :-1] + d / 2, outline, cutouts)
    xb = node[:-1, :] & node[1:, :] & mx
    yb = node[:, :-1] & node[:, 1:] & my
    if not exact:
        return node, xb, yb
    from . import raster
    pa, pb = raster.ring_edges(outline, cutouts)
    # an x strip (i, j) crosses the border x = (i + 1/2) d, |y - j d| <= d / 2; a y strip the border y = (j + 1/2) d
    cx = raster.line_cover(pa[:, 0], pa[:, 1], pb[:, 0], pb[:, 1], d / 2, d, nx - 1, 0.0, d, ny) / d
    cy = raster.line_cover(pa[:, 1], pa[:, 0], pb[:, 1], pb[:, 0], d / 2, d, ny - 1, 0.0, d, nx).T / d
    zx, zy = np.zeros(xb.shape), np.zeros(yb.shape)
    wx, ox = raster.strip_widths(xb, cx, zx, zx, d)
    wy, oy = raster.strip_widths(yb, cy, zy, zy, d)
    return node, xb, yb, {"wx": np.where(xb, wx, 1.0), "wy": np.where(yb, wy, 1.0), "ox": ox, "oy": oy}


def rect_polygon(cx: float, cy: float, length: float, width: float, angle: float) -> np.ndarray:
    """A rectangle centred at (cx, cy), `length` along direction `angle` (rad), `width` across."""
    u = np.array([math.cos(angle), math.sin(angle)])
    v = np.array([-u[1], u[0]])
    c = np.array([cx, cy])
    a, b = 0.5 * length, 0.5 * width
    return np.array([c - a * u - b * v, c + a * u - b * v, c + a * u + b * v, c - a * u + b * v])


# ------------------------------------------------------------------------------------------ board
@dataclass
class Layer:
    name: str
    z: float
    thickness: float
    node: np.ndarray
    xb: np.ndarray
    yb: np.ndarray
    # strips narrower than the pitch (the reference Grid's wx / wy, ox / oy, rx / ry: width and centre offset as
    # fractions of the pitch, the resistance's width; None: every strip full and centred)
    widths: Optional[dict] = None
    # a sub-grid raster's cells (the reference Grid's fill / area / label: each cell's copper fraction, each node's
    # measured copper, each node's net; None: whole cells, no measured copper, one net)
    fill: Optional[np.ndarray] = None
    area: Optional[np.ndarray] = None
    label: Optional[np.ndarray] = None


@dataclass
class Pair:
    upper: int
    lower: int
    c_per_area: float
    tan_delta: float = 0.02


@dataclass
class BranchSpec:
    """Lumped branch a -> b, impedance R + jwL (+ 1/(jwC) when C > 0)."""
    a: tuple
    b: tuple
    R: float
    L: float
    C: float = 0.0
    kind: str = "part"
    radius: float = 1.5e-4

    def z(self, f: float) -> complex:
        w = 2 * math.pi * f
        z = complex(self.R, w * self.L)
        if self.C > 0:
            z += 1.0 / (1j * w * self.C)
        return z


@dataclass
class Net:
    """Known signal path: rows (ax, ay, az, bx, by, bz, width, i), metres relative to node (0, 0)."""
    segments: np.ndarray
    driver: tuple
    receiver: tuple
    trace_t: float = 35e-6


@dataclass
class Board:
    name: str
    d: float                      # pitch, metres
    nx: int
    ny: int
    layers: list
    pairs: list = field(default_factory=list)
    branches: list = field(default_factory=list)
    nets: list = field(default_factory=list)
    freqs: np.ndarray = field(default_factory=lambda: np.zeros(0))
    precond: str = "diag"
    tol: float = 1e-10
    restart: int = 50
    sigma: float = SIGMA_CU
    screen: bool = False          # split layers with copper above and below into two face sheets

    # -- flat arrays (fixtures, the C-ABI) -----------------------------------------------------------
    def to_arrays(self) -> dict:
        out = {"name": np.array(self.name), "d": np.float64(self.d), "nx": np.int64(self.nx),
               "ny": np.int64(self.ny), "precond": np.array(self.precond), "tol": np.float64(self.tol),
               "restart": np.int64(self.restart), "sigma": np.float64(self.sigma),
               "freqs": np.asarray(self.freqs, float),
               "layer_z": np.array([l.z for l in self.layers]), "layer_t": np.array([l.thickness for l in self.layers]),
               "layer_node": np.stack([l.node for l in self.layers]), "layer_xb": np.stack([l.xb for l in self.layers]),
               "layer_yb": np.stack([l.yb for l in self.layers]),
               "pairs": np.array([[p.upper, p.lower, p.c_per_area, p.tan_delta] for p in self.pairs], float).reshape(-1, 4),
               "branch_ab": np.array([[*b.a, *b.b] for b in self.branches], np.int64).reshape(-1, 6),
               "branch_rlc": np.array([[b.R, b.L, b.C, b.radius] for b in self.branches], float).reshape(-1, 4),
               "branch_via": np.array([b.kind == "via" for b in self.branches], bool),
               "net_count": np.int64(len(self.nets)), "screen": np.bool_(self.screen)}
        for k, l in enumerate(self.layers):
            for key, v in (l.widths or {}).items():
                out[f"layer{k}_{key}"] = np.asarray(v, float)
            for key in CELL_KEYS:
                if getattr(l, key) is not None:
                    out[f"layer{k}_{key}"] = np.asarray(getattr(l, key), np.int64 if key == "label" else float)
        for n, net in enumerate(self.nets):
            out[f"net{n}_seg"] = net.segments
            out[f"net{n}_ends"] = np.array([*net.driver, *net.receiver], np.int64)
            out[f"net{n}_trace_t"] = np.float64(net.trace_t)
        return out

    @staticmethod
    def from_arrays(a) -> "Board":
        layers = [Layer(f"L{k}", float(a["layer_z"][k]), float(a["layer_t"][k]), a["layer_node"][k].astype(bool),
                        a["layer_xb"][k].astype(bool), a["layer_yb"][k].astype(bool)) for k in range(len(a["layer_z"]))]
        files = a.files if hasattr(a, "files") else list(a.keys())
        for k, l in enumerate(layers):
            w = {key: np.asarray(a[f"layer{k}_{key}"], float) for key in WIDTH_KEYS if f"layer{k}_{key}" in files}
            l.widths = w or None
            for key in CELL_KEYS:
                if f"layer{k}_{key}" in files:
                    setattr(l, key, np.asarray(a[f"layer{k}_{key}"]))
        pairs = [Pair(int(p[0]), int(p[1]), float(p[2]), float(p[3])) for p in a["pairs"]]
        branches = [BranchSpec(tuple(int(v) for v in ab[:3]), tuple(int(v) for v in ab[3:]), float(r[0]), float(r[1]),
                               float(r[2]), "via" if via else "part", float(r[3]))
                    for ab, r, via in zip(a["branch_ab"], a["branch_rlc"], a["branch_via"])]
        nets = []
        for n in range(int(a["net_count"])):
            e = a[f"net{n}_ends"]
            nets.append(Net(np.asarray(a[f"net{n}_seg"], float), tuple(int(v) for v in e[:3]),
                            tuple(int(v) for v in e[3:]), float(a[f"net{n}_trace_t"])))
        return Board(str(a["name"]), float(a["d"]), int(a["nx"]), int(a["ny"]), layers, pairs, branches, nets,
                     np.asarray(a["freqs"], float), str(a["precond"]), float(a["tol"]), int(a["restart"]),
                     float(a["sigma"]), bool(a["screen"]) if "screen" in files else False)


def _full_layer(name, z, t, nx, ny, d, cutouts=()):
    """A plane whose outline reaches half a pitch beyond the grid (every grid node inside), minus cut-outs."""
    h = 0.5 * d
    outline = np.array([[-h, -h], [(nx - 1) * d + h, -h], [(nx - 1) * d + h, (ny - 1) * d + h], [-h, (ny - 1) * d + h]])
    node, xb, yb = raster_layer(nx, ny, d, outline, list(cutouts))
    return Layer(name, z, t, node, xb, yb)


def _segments(points: list, z_sig: float, z_face: float, width: float) -> np.ndarray:
    """Filaments: up from the plane's face at the first point, along the walk at z_sig, down at the last."""
    rows = []
    p0, p1 = points[0], points[-1]
    rows.append([p0[0], p0[1], z_face, p0[0], p0[1], z_sig, width, 1.0])
    for a, b in zip(points[:-1], points[1:]):
        rows.append([a[0], a[1], z_sig, b[0], b[1], z_sig, width, 1.0])
    rows.append([p1[0], p1[1], z_sig, p1[0], p1[1], z_face, width, 1.0])
    return np.array(rows, float)


def plain_plane(n: int = 96, d_mm: float = 0.5, f: float = 1e8) -> Board:
    """One solid plane, a straight trace 0.2 mm above its top face from (10, 48) to (86, 48)."""
    d = d_mm * 1e-3
    t = 35e-6
    layer = _full_layer("GND", 0.0, t, n, n, d)
    i0, i1, j = round(10 * n / 96), round(86 * n / 96), n // 2
    z_face, z_sig = 0.5 * t, 0.5 * t + 0.2e-3
    pts = [(i0 * d, j * d), (i1 * d, j * d)]
    net = Net(_segments(pts, z_sig, z_face, 0.2e-3), (0, i0, j), (0, i1, j))
    return Board("plain_plane", d, n, n, [layer], nets=[net], freqs=np.array([f]), precond="diag",
                 tol=1e-10, restart=50)


def _manhattan_walk(rng, start, mid, end, nseg: int, lo: int, hi_x: int, hi_y: int) -> list:
    """Cell coordinates of an axis-aligned walk start -> mid -> end with about `nseg` segments; each leg
    wanders with random steps biased toward its goal and closes with one x and one y move."""
    pts = [tuple(start)]
    legs = [(mid, nseg // 2), (end, nseg - nseg // 2)]
    axis = 0
    for goal, n in legs:
        cur = list(pts[-1])
        for _ in range(max(n - 2, 0)):
            gap = goal[axis] - cur[axis]
            step = int(rng.integers(1, 9)) * (1 if rng.random() < 0.5 + 0.35 * np.sign(gap) else -1)
            nxt = cur.copy()
            nxt[axis] = int(np.clip(cur[axis] + step, lo, (hi_x if axis == 0 else hi_y)))
            if nxt[axis] != cur[axis]:
                cur = nxt
                pts.append(tuple(cur))
            axis ^= 1
        for ax in (axis, axis ^ 1):
            if cur[ax] != goal[ax]:
                cur = cur.copy()
                cur[ax] = goal[ax]
                pts.append(tuple(cur))
        axis = 0
    return pts


def slotted_pair(n: int = 256, d_mm: float = 0.25, n_nets: int = 8, n_freq: int = 32, seed: int = 2,
                 f_lo: float = 1e6, f_hi: float = 1e9, seg_range=(20, 60)) -> Board:
    """Sig/GND/PWR/Sig with a seeded 1 mm slot across 60 % of the GND plane and random-walk nets on the top
    signal layer, each crossing the slot, returning in GND (driver/receiver vias at the walk's ends)."""
    rng = np.random.default_rng(seed)
    d = d_mm * 1e-3
    t = 35e-6
    side = (n - 1) * d
    length = 0.6 * n * d
    cx, cy = side * rng.uniform(0.4, 0.6), side * rng.uniform(0.4, 0.6)
    ang = rng.uniform(0, math.pi)
    slot = rect_polygon(cx, cy, length, 1e-3, ang)
    gnd = _full_layer("GND", 0.0, t, n, n, d, [slot])
    pwr = _full_layer("PWR", -(1.0e-3 + t), t, n, n, d)
    pair = Pair(0, 1, EPS0 * 4.3 / 1.0e-3, 0.02)
    z_face, z_sig = 0.5 * t, 0.2e-3 + t
    u = np.array([math.cos(ang), math.sin(ang)])
    v = np.array([-u[1], u[0]])
    margin = max(4, n // 32)
    nets = []
    for k in range(n_nets):
        for _ in range(1000):
            along = rng.uniform(-0.35, 0.35) * length
            off = rng.uniform(0.15, 0.4) * side
            s = np.array([cx, cy]) + along * u - off * v
            e = np.array([cx, cy]) + rng.uniform(-0.35, 0.35) * length * u + rng.uniform(0.15, 0.4) * side * v
            m = np.array([cx, cy]) + rng.uniform(-0.3, 0.3) * length * u
            cs, ce, cm = (np.round(p / d).astype(int) for p in (s, e, m))
            ok = all(margin <= c[0] < n - margin and margin <= c[1] < n - margin for c in (cs, ce, cm))
            if ok and gnd.node[cs[0], cs[1]] and gnd.node[ce[0], ce[1]]:
                break
        nseg = int(rng.integers(seg_range[0], seg_range[1] + 1))
        cells = _manhattan_walk(rng, cs, cm, ce, nseg, margin, n - 1 - margin, n - 1 - margin)
        pts = [(c[0] * d, c[1] * d) for c in cells]
        nets.append(Net(_segments(pts, z_sig, z_face, 0.15e-3), (0, int(cs[0]), int(cs[1])),
                        (0, int(ce[0]), int(ce[1]))))
    freqs = np.logspace(math.log10(f_lo), math.log10(f_hi), n_freq)
    return Board("slotted_pair", d, n, n, [gnd, pwr], [pair], [], nets, freqs, precond="sheet", tol=1e-10,
                 restart=50)


def small_pair(seed: int = 5) -> Board:
    """A reduced slotted plane pair (40 x 36 at 0.5 mm) with a decoupling part and a stitching via."""
    rng = np.random.default_rng(seed)
    nx, ny, d = 40, 36, 0.5e-3
    t = 35e-6
    slot = rect_polygon(20 * d, 17 * d, 0.6 * 36 * d, 1.0e-3, rng.uniform(0.2, 1.2))
    gnd = _full_layer("GND", 0.0, t, nx, ny, d, [slot])
    pwr = _full_layer("PWR", -(0.5e-3 + t), 18e-6, nx, ny, d)
    pair = Pair(0, 1, EPS0 * 4.3 / 0.5e-3, 0.02)
    # a decap (ESR 20 mohm, ESL 0.5 nH, 100 nF) between GND and PWR, and one via joining them elsewhere
    decap = BranchSpec((0, 6, 30), (1, 6, 30), 0.02, 0.5e-9, 100e-9, "part")
    via_len = 0.5e-3 + t
    via = BranchSpec((0, 33, 4), (1, 33, 4), via_len / (SIGMA_CU * math.pi * 2 * 1.5e-4 * 25e-6), 2.0e-10, 0.0, "via",
                     1.5e-4)
    z_face, z_sig = 0.5 * t, 0.2e-3 + t
    nets = []
    for (s, m, e) in (((6, 6), (20, 17), (33, 29)), ((34, 8), (18, 18), (8, 26))):
        cells = _manhattan_walk(rng, s, m, e, 12, 2, nx - 3, ny - 3)
        pts = [(c[0] * d, c[1] * d) for c in cells]
        nets.append(Net(_segments(pts, z_sig, z_face, 0.15e-3), (0, *s), (0, *e)))
    return Board("small_pair", d, nx, ny, [gnd, pwr], [pair], [decap, via], nets, np.array([1e6, 1e8, 1e9]),
                 precond="sheet", tol=1e-10, restart=50)


def small_stack3(seed: int = 9) -> Board:
    """Three planes (non-square 30 x 44 at 0.4 mm) with polygon cut-outs, stitching vias, diag precond."""
    rng = np.random.default_rng(seed)
    nx, ny, d = 30, 44, 0.4e-3
    t = 35e-6
    layers = []
    zs = [0.0, -(0.3e-3 + t), -(1.5e-3 + 2 * t)]
    for k, z in enumerate(zs):
        cuts = []
        for _ in range(int(rng.integers(0, 3))):
            c = np.array([rng.uniform(0.2, 0.8) * (nx - 1) * d, rng.uniform(0.2, 0.8) * (ny - 1) * d])
            nv = int(rng.integers(3, 7))
            ang = np.sort(rng.uniform(0, 2 * math.pi, nv))
            rad = rng.uniform(0.6e-3, 1.6e-3, nv)
            cuts.append(c + np.stack([rad * np.cos(ang), rad * np.sin(ang)], 1))
        layers.append(_full_layer(f"L{k}", z, t, nx, ny, d, cuts))
    branches = []
    for _ in range(6):
        i, j = int(rng.integers(2, nx - 2)), int(rng.integers(2, ny - 2))
        k0, k1 = 0, int(rng.integers(1, 3))
        if layers[k0].node[i, j] and layers[k1].node[i, j]:
            length = abs(zs[k0] - zs[k1])
            branches.append(BranchSpec((k0, i, j), (k1, i, j), length / (SIGMA_CU * math.pi * 2 * 1.5e-4 * 25e-6),
                                       2e-10 * length / 1e-3, 0.0, "via", 1.5e-4))
    z_face, z_sig = 0.5 * t, 0.15e-3 + t
    ends = [c for c in ((3, 5), (26, 38), (4, 40), (25, 4), (15, 2), (15, 41)) if layers[0].node[c]]
    s, e = ends[0], ends[1]
    cells = _manhattan_walk(rng, s, (15, 22), e, 10, 2, nx - 3, ny - 3)
    pts = [(c[0] * d, c[1] * d) for c in cells]
    nets = [Net(_segments(pts, z_sig, z_face, 0.2e-3), (0, *s), (0, *e))]
    return Board("small_stack3", d, nx, ny, layers, [], branches, nets, np.array([3e6, 3e8]), precond="diag",
                 tol=1e-10, restart=50)


def random_board(seed: int, side=(24, 48), n_layers=(2, 6), n_nets=(1, 2), n_freq: int = 2, slots: bool = False,
                 cut_max: int = 8, pitch_mm: Optional[float] = None) -> Board:
    """A seeded board drawn like the uneven-batch workload (sides, pitch, 2-6 plane layers with gaps
    U[0.1, 1.5] mm, 0-8 polygon cut-outs of 3-8 vertices per layer, stitching vias at a Poisson density of
    0-4 per cm2, random-walk nets, log-spaced frequencies in [1 MHz, 1 GHz]), with the raster sides drawn from
    `side` (small enough for the FP64 oracle); `slots`: also one straight slot per layer (the largest
    instance's layers); `pitch_mm`: this pitch instead of the drawn one.  The nets' return nodes are on the top
    plane and connected there."""
    rng = np.random.default_rng(seed)
    nx, ny = (int(rng.integers(side[0], side[1] + 1)) for _ in range(2))
    d = float(rng.uniform(0.2, 0.5)) * 1e-3
    if pitch_mm is not None:
        d = pitch_mm * 1e-3
    t = 35e-6
    nl = int(rng.integers(n_layers[0], n_layers[1] + 1))
    zs = [0.0]
    for _ in range(nl - 1):
        zs.append(zs[-1] - (float(rng.uniform(0.1, 1.5)) * 1e-3 + t))
    W, H = (nx - 1) * d, (ny - 1) * d
    layers = []
    for k, z in enumerate(zs):
        cuts = []
        for _ in range(int(rng.integers(0, cut_max + 1))):
            c = np.array([rng.uniform(0.15, 0.85) * W, rng.uniform(0.15, 0.85) * H])
            nv = int(rng.integers(3, 9))
            ang = np.sort(rng.uniform(0, 2 * math.pi, nv))
            rad = rng.uniform(0.03, 0.09, nv) * min(W, H)
            cuts.append(c + np.stack([rad * np.cos(ang), rad * np.sin(ang)], 1))
        if slots:
            cuts.append(rect_polygon(rng.uniform(0.3, 0.7) * W, rng.uniform(0.3, 0.7) * H, 0.5 * min(W, H),
                                     2.2 * d, rng.uniform(0, math.pi)))
        layers.append(_full_layer(f"L{k}", z, t, nx, ny, d, cuts))
    branches = []
    lam = float(rng.uniform(0.0, 4.0)) * (W * H * 1e4)          # vias on the board (density per cm2)
    for _ in range(int(rng.poisson(lam))):
        i, j = int(rng.integers(1, nx - 1)), int(rng.integers(1, ny - 1))
        k0, k1 = sorted(int(v) for v in rng.choice(nl, 2, replace=False))
        if layers[k0].node[i, j] and layers[k1].node[i, j]:
            length = abs(zs[k0] - zs[k1])
            branches.append(BranchSpec((k0, i, j), (k1, i, j), length / (SIGMA_CU * math.pi * 2 * 1.5e-4 * 25e-6),
                                       2e-10 * length / 1e-3, 0.0, "via", 1.5e-4))
    z_face, z_sig = 0.5 * t, 0.15e-3 + t
    top = layers[0].node
    lab = _labels(top, layers[0].xb, layers[0].yb)
    nets = []
    for _ in range(int(rng.integers(n_nets[0], n_nets[1] + 1))):
        for _try in range(200):
            s = (int(rng.integers(2, nx - 2)), int(rng.integers(2, ny - 2)))
            e = (int(rng.integers(2, nx - 2)), int(rng.integers(2, ny - 2)))
            if top[s] and top[e] and lab[s] == lab[e] and abs(s[0] - e[0]) + abs(s[1] - e[1]) > min(nx, ny) // 3:
                break
        else:
            raise RuntimeError("no connected pair of return nodes on the top plane")
        mid = ((s[0] + e[0]) // 2, (s[1] + e[1]) // 2)
        cells = _manhattan_walk(rng, s, mid, e, int(rng.integers(4, 12)), 2, nx - 3, ny - 3)
        pts = [(c[0] * d, c[1] * d) for c in cells]
        nets.append(Net(_segments(pts, z_sig, z_face, 0.15e-3), (0, *s), (0, *e)))
    if isinstance(n_freq, tuple):           # a count drawn from the range, log-spaced over the band
        freqs = np.geomspace(1e6, 1e9, int(rng.integers(n_freq[0], n_freq[1] + 1)))
    else:
        freqs = np.sort(np.exp(rng.uniform(math.log(1e6), math.log(1e9), n_freq)))
    return Board(f"random_{seed}", d, nx, ny, layers, [], branches, nets, freqs, precond="diag", tol=1e-10,
                 restart=50)


def uneven_board(seed: int, tol: float = 1e-8) -> Board:
    """One board of the uneven-batch workload at its full sizes: raster sides U[64, 512] per axis, pitch
    U[0.2, 0.5] mm, 2-6 plane layers with gaps U[0.1, 1.5] mm, 0-8 polygon cut-outs of 3-8 vertices per layer,
    stitching vias at a Poisson density of 0-4 per cm2, 1-16 random-walk nets and 4-16 log-spaced frequencies
    from 1 MHz to 1 GHz; solved to `tol`."""
    b = random_board(10_000 + seed, side=(64, 512), n_layers=(2, 6), n_nets=(1, 16), n_freq=(4, 16))
    b.name, b.tol = f"uneven_{seed}", tol
    return b


def largest_board(n: int = 1024, pitch_mm: float = 0.1, n_nets: int = 32, n_freq: int = 64, seed: int = 5,
                  tol: float = 1e-8) -> Board:
    """The largest single instance: six plane layers of n x n nodes at pitch_mm (1024 x 1024 at 0.1 mm: a
    10 cm board, ~12.6 M strips), cut-outs and a slot on every layer, stitching vias, n_nets random-walk nets
    and n_freq log-spaced frequencies from 1 MHz to 1 GHz."""
    b = random_board(seed, side=(n, n), n_layers=(6, 6), n_nets=(n_nets, n_nets), n_freq=(n_freq, n_freq),
                     slots=True, cut_max=3, pitch_mm=pitch_mm)
    b.name, b.tol = f"largest_{n}", tol
    return b


def six_sheet(seed: int = 21) -> Board:
    """The largest instance's shape at oracle size: six plane layers, cut-outs and a slot on every layer."""
    return random_board(seed, side=(28, 40), n_layers=(6, 6), n_nets=(1, 2), slots=True, cut_max=3)


def _labels(mask: np.ndarray, xb: np.ndarray, yb: np.ndarray) -> np.ndarray:
    """Connected components of a layer's nodes joined by its x / y strips; -1 off copper."""
    lab = -np.ones(mask.shape, np.int64)
    nxx, nyy = mask.shape
    cur = 0
    for i0 in range(nxx):
        for j0 in range(nyy):
            if not mask[i0, j0] or lab[i0, j0] >= 0:
                continue
            stack = [(i0, j0)]
            lab[i0, j0] = cur
            while stack:
                i, j = stack.pop()
                nbrs = []
                if i + 1 < nxx and xb[i, j]:
                    nbrs.append((i + 1, j))
                if i > 0 and xb[i - 1, j]:
                    nbrs.append((i - 1, j))
                if j + 1 < nyy and yb[i, j]:
                    nbrs.append((i, j + 1))
                if j > 0 and yb[i, j - 1]:
                    nbrs.append((i, j - 1))
                for a, b in nbrs:
                    if mask[a, b] and lab[a, b] < 0:
                        lab[a, b] = cur
                        stack.append((a, b))
            cur += 1
    return lab


WIDTH_KEYS = ("wx", "wy", "ox", "oy", "rx", "ry")
CELL_KEYS = ("fill", "area", "label")


def plane_pair_line(length_mm: float, w: float = 10e-3, h: float = 0.2e-3, t: float = 35e-6, d: float = 0.4e-3,
                    f=(1e6, 1e8)) -> Board:
    """A parallel-plate line (the reference's plane_pair_line, tests/boardgen.py:1149-1178): two strips `w` wide
    and `length_mm` long, copper `t` thick, `h` of dielectric between their faces (layer heights at the foils'
    centres, h + t apart), on pitch d.  A row of ten shorts 1 mm apart across the far end (a capacitor's short
    model: 1 uOhm, 1 fH), fed between the strips near the other end: the one net has no trace, its receiver on the
    upper strip (+1 A in) and its driver on the lower one, so its loop impedance is the port's."""
    nx, ny = int(round(length_mm * 1e-3 / d)), int(round(w / d))
    node = np.ones((nx, ny), bool)
    layers = [Layer(name, z, t, node.copy(), np.ones((nx - 1, ny), bool), np.ones((nx, ny - 1), bool))
              for name, z in (("VDD", 0.0), ("GND", -(h + t)))]
    n = 10
    shorts = [BranchSpec((0, nx - 2, j), (1, nx - 2, j), 1e-6, 1e-15) for j in
              (int((k + 0.5) * w / n / d) for k in range(n))]
    feed = ny // 2
    net = Net(np.zeros((0, 8)), (1, 2, feed), (0, 2, feed))
    return Board(f"plane_pair_line{length_mm:g}", d, nx, ny, layers, branches=shorts, nets=[net],
                 freqs=np.asarray(f, float), precond="sheet", tol=1e-8, restart=50)


def microstrip(slot: float = 0.0, edge_split: bool = False, full_cut: bool = False, f=(1e8,)) -> Board:
    """A 40 x 20 mm plane (35 um copper at z = 0) on 0.25 mm pitch under a 0.2 mm trace 0.5 mm above it, from
    (5, 10) to (35, 10) mm, dropping to the plane at both ends (the reference's analytic cases, tests/
    test_solver.py:19-30): slot = a 1 mm wide slot of that length (mm) across the trace at x = 20 mm;
    edge_split = a 1 mm cut from y = 4 mm to the plane's edge; full_cut = a cut across the whole plane."""
    d, t, H, W = 0.25e-3, 35e-6, 0.5e-3, 0.2e-3
    nx, ny = 161, 81
    outline = np.array([[0.0, 0.0], [40e-3, 0.0], [40e-3, 20e-3], [0.0, 20e-3]])
    cuts = []

    def box(x0, y0, x1, y1):
        return np.array([[x0, y0], [x1, y0], [x1, y1], [x0, y1]]) * 1e-3
    if slot:
        cuts.append(box(19.5, 10 - slot / 2, 20.5, 10 + slot / 2))
    if edge_split:
        cuts.append(box(19.5, 4, 20.5, 20.1))
    if full_cut:
        cuts.append(box(19.5, -1, 20.5, 21))
    node, xb, yb = raster_layer(nx, ny, d, outline, cuts)
    layer = Layer("GND", 0.0, t, node, xb, yb)
    i0, i1, j = 20, 140, 40
    pts = [(i0 * d, j * d), (i1 * d, j * d)]
    net = Net(_segments(pts, H, 0.0, W), (0, i0, j), (0, i1, j))
    return Board("microstrip", d, nx, ny, [layer], nets=[net], freqs=np.asarray(f, float), precond="diag",
                 tol=1e-5, restart=50)


def necked_faces(seed: int = 23) -> Board:
    """faces_stack3 ('sheet' preconditioner) with strips narrower than the pitch on the split middle layer and
    on the top one: the split layer's faces share their copper's corrections (PlaneStack._twin_corrections,
    peec.py:1822-1843) and its face blocks carry them (peec.py:2497-2503)."""
    rng = np.random.default_rng(seed)
    b = faces_stack3("sheet")
    b.name = "necked_faces"
    for k in (0, 1):
        l = b.layers[k]
        nx, ny = l.node.shape
        wx, wy = np.ones((nx - 1, ny)), np.ones((nx, ny - 1))
        ox, oy = np.zeros((nx - 1, ny)), np.zeros((nx, ny - 1))
        rx, ry = np.zeros((nx - 1, ny)), np.zeros((nx, ny - 1))
        xs, ys = np.argwhere(l.xb), np.argwhere(l.yb)
        for (i, j) in xs[rng.choice(len(xs), size=10, replace=False)]:
            wx[i, j] = rng.uniform(0.3, 0.9)
            ox[i, j] = rng.uniform(-0.5, 0.5) * (1 - wx[i, j])
        for (i, j) in ys[rng.choice(len(ys), size=10, replace=False)]:
            wy[i, j] = rng.uniform(0.3, 0.9)
            oy[i, j] = rng.uniform(-0.5, 0.5) * (1 - wy[i, j])
        i, j = xs[0]
        rx[i, j] = 0.8 * wx[i, j] if wx[i, j] < 1 else 0.7
        l.widths = {"wx": wx, "wy": wy, "ox": ox, "oy": oy, "rx": rx, "ry": ry}
    return b


def faces_stack3(precond: str = "diag") -> Board:
    """small_stack3 with screening on: its middle plane has copper above and below, so it is split into two
    face sheets (PlaneStack._faces, peec.py:1658-1697): four current sheets on three layers."""
    b = small_stack3()
    b.name = f"faces_stack3_{precond}"
    b.precond = precond
    b.screen = True
    return b


def necked_pair(seed: int = 17) -> Board:
    """A plane pair (40 x 36 at 0.5 mm) whose PWR plane has an island joined to the rest by a neck narrower
    than the pitch, with seeded narrow, off-centre and series-narrowed strips along the moat (the exact-copper
    raster's wx / wy, ox / oy, rx / ry), a decoupling part on the island and two nets crossing the GND slot."""
    rng = np.random.default_rng(seed)
    b = small_pair(seed=5)
    b.name = "necked_pair"
    pwr = b.layers[1]
    node = pwr.node.copy()
    i0, i1, j0, j1 = 25, 37, 21, 33                 # the moat: one cell wide around the island
    node[i0, j0:j1 + 1] = False
    node[i1, j0:j1 + 1] = False
    node[i0:i1 + 1, j0] = False
    node[i0:i1 + 1, j1] = False
    node[i0, 26:28] = True                          # the neck through the moat's left side
    xb = node[:-1, :] & node[1:, :]
    yb = node[:, :-1] & node[:, 1:]
    nx, ny = node.shape
    wx, wy = np.ones((nx - 1, ny)), np.ones((nx, ny - 1))
    ox, oy = np.zeros((nx - 1, ny)), np.zeros((nx, ny - 1))
    rx, ry = np.zeros((nx - 1, ny)), np.zeros((nx, ny - 1))
    for i in (i0 - 1, i0):                          # the neck's x strips: 0.35-0.45 of the pitch
        for j in (26, 27):
            wx[i, j] = rng.uniform(0.35, 0.45)
            ox[i, j] = 0.1 if j == 26 else -0.1
    wy[i0, 26] = 0.5
    rx[i0 - 1, 26] = 0.8 * wx[i0 - 1, 26]           # a change of width along the strip, in series
    rx[i0, 27] = 0.9 * wx[i0, 27]
    # strips along the moat's outside: partly covered borders
    edge_y = [(i0 - 1, j) for j in range(j0, j1) if yb[i0 - 1, j] and j not in (25, 26, 27)]
    for q in rng.choice(len(edge_y), size=min(8, len(edge_y)), replace=False):
        i, j = edge_y[q]
        wy[i, j] = rng.uniform(0.55, 0.95)
        oy[i, j] = rng.uniform(-0.5, 0.5) * (1 - wy[i, j])
    edge_x = [(i, j0 - 1) for i in range(i0, i1) if xb[i, j0 - 1]]
    for q in rng.choice(len(edge_x), size=min(4, len(edge_x)), replace=False):
        i, j = edge_x[q]
        wx[i, j] = rng.uniform(0.6, 0.95)
        ox[i, j] = rng.uniform(-0.5, 0.5) * (1 - wx[i, j])
    ry[i0 - 1, j0 + 2] = 0.7 if yb[i0 - 1, j0 + 2] else 0.0
    b.layers[1] = Layer(pwr.name, pwr.z, pwr.thickness, node, xb, yb,
                        {"wx": wx, "wy": wy, "ox": ox, "oy": oy, "rx": rx, "ry": ry})
    # the decoupling part moves onto the island (the small pair's other branches stay)
    b.branches = [BranchSpec((0, 30, 27), (1, 30, 27), 0.02, 0.5e-9, 100e-9, "part")] + b.branches[1:]
    b.freqs = np.array([1e6, 1e8, 1e9])
    return b


def track_rail(length_mm: float, width_mm: float, angle: float = 0.0, dy: float = 0.0, d_mm: float = 0.5,
               sub: int = 4) -> Board:
    """A copper track `width_mm` wide and `length_mm` long at `angle` degrees between two 1 x 1 mm pads (the
    reference's track-width rail, tests/test_track_width.py:58-70: one layer, no plane), rasterised with its
    exact widths (raster.build_layer at sub-grid `sub`, the centreline forced as a track); `dy` moves it off the
    grid's rows.  Its one net has no trace and its ends at the pads' nodes, for the DC resistance at 0 Hz."""
    from . import raster
    a = math.radians(angle)
    x0, y0 = 3.0, 3.0 + dy
    x1, y1 = x0 + length_mm * math.cos(a), y0 + length_mm * math.sin(a)
    h = width_mm / 2
    u = np.array([-0.5, 0.5, 0.5, length_mm - 0.5, length_mm - 0.5, length_mm + 0.5, length_mm + 0.5,
                  length_mm - 0.5, length_mm - 0.5, 0.5, 0.5, -0.5])
    v = np.array([-0.5, -0.5, -h, -h, -0.5, -0.5, 0.5, 0.5, h, h, 0.5, 0.5])
    outline = np.stack([x0 + math.cos(a) * u - math.sin(a) * v, y0 + math.sin(a) * u + math.cos(a) * v], 1)
    bbox = (0.0, 0.0, x1 + 3.0, max(y1 + 3.0, 6.0))
    g = raster.build_layer({"PWR": [(outline, [])]}, bbox, d_mm,
                           lines={"PWR": [(np.array([[x0, y0], [x1, y1]]), width_mm)]}, sub=sub)
    grid_nodes = np.argwhere(g.node)

    def node_at(x, y):
        k = int(np.argmin((grid_nodes[:, 0] * d_mm - x) ** 2 + (grid_nodes[:, 1] * d_mm - y) ** 2))
        return (0, int(grid_nodes[k, 0]), int(grid_nodes[k, 1]))
    layer = Layer("F", 0.0, 35e-6, g.node, g.xb, g.yb, g.widths(), g.fill, g.area, g.label)
    net = Net(np.zeros((0, 8)), node_at(x0, y0), node_at(x1, y1))
    return Board(f"track_rail{length_mm:g}", d_mm * 1e-3, g.nx, g.ny, [layer], nets=[net], freqs=np.array([0.0]),
                 precond="diag", tol=1e-10, restart=50)


def routed_pair(sub: int = 4) -> Board:
    """A plane pair rasterised from polygons by raster.build_layer (GroundTruth's build_grid) at sub-grid `sub`,
    with the copper's exact widths: a GND pour (a slanted slot, a square hole, a notched corner with a pad in it
    joined to the pour by a 0.25 mm corridor, its track's centreline forced) over a PWR plane with a cut-out;
    0.5 mm pitch, 40 x 36 nodes, a decoupling part and a via, two nets crossing the slot.  The copper's ragged
    edges give strips narrower than the pitch all around (wx / wy, ox / oy, rx / ry), cells partly covered (their
    plane-pair capacitance the facing share) and measured node areas."""
    from . import raster
    d_mm, t, h = 0.5, 35e-6, 0.2e-3
    bbox = (0.0, 0.0, 19.5, 17.5)
    pour = (np.array([[0.2, 0.3], [19.3, 0.3], [19.3, 17.2], [4.1, 17.2], [4.1, 13.6], [1.725, 13.6],
                      [1.725, 15.1], [2.3, 15.1], [2.3, 16.4], [0.9, 16.4], [0.9, 15.1], [1.475, 15.1],
                      [1.475, 13.6], [0.2, 13.6]]),
            [rect_polygon(10.0, 8.6, 8.0, 0.6, math.radians(30.0)),
             np.array([[14.3, 3.1], [15.6, 3.1], [15.6, 4.4], [14.3, 4.4]])])
    gnd = raster.build_layer({"GND": [pour]}, bbox, d_mm,
                             lines={"GND": [(np.array([[1.6, 15.7], [1.6, 13.0]]), 0.25)]}, sub=sub)
    plane = (np.array([[0.1, 0.1], [19.4, 0.1], [19.4, 17.4], [0.1, 17.4]]),
             [np.array([[5.2, 2.3], [7.9, 2.3], [7.9, 4.1], [5.2, 4.1]])])
    pwr = raster.build_layer({"PWR": [plane]}, bbox, d_mm, sub=sub)
    layers = [Layer(name, z, t, g.node, g.xb, g.yb, g.widths(), g.fill, g.area, g.label)
              for name, z, g in (("GND", 0.0, gnd), ("PWR", -(h + t), pwr))]
    d = d_mm * 1e-3
    pairs = [Pair(0, 1, EPS0 * 4.4 / h)]
    branches = [BranchSpec((0, 30, 26), (1, 30, 26), 0.02, 0.5e-9, 100e-9, "part"),
                BranchSpec((0, 8, 30), (1, 8, 30), 1e-3, 0.3e-9, 0.0, "via", 1.5e-4)]
    nets = []
    for (i0, j0), (i1, j1) in (((6, 5), (32, 12)), ((12, 24), (33, 6))):
        pts = [(i0 * d, j0 * d), (i0 * d, j1 * d), (i1 * d, j1 * d)]
        nets.append(Net(_segments(pts, 0.3e-3, 0.0, 0.2e-3), (0, i0, j0), (0, i1, j1)))
    return Board("routed_pair", d, gnd.nx, gnd.ny, layers, pairs, branches, nets, np.array([1e6, 1e8, 1e9]),
                 precond="sheet", tol=1e-10, restart=50)


def what_if_base(n: int = 512, d_mm: float = 0.2, n_nets: int = 12, n_freq: int = 16, seed: int = 4,
                 slot: bool = True, n_decap: int = 8) -> Board:
    """The interactive what-if workload's base board: 4-layer Sig/GND/PWR/Sig at d_mm pitch, the GND/PWR pair
    solved (sheet preconditioner), PWR split into two islands by a 1 mm gap across the board, a seeded 1 mm
    GND slot across 60 % of the board (slot=False: the same board with the slot filled, the "toggle the slot"
    edit), n_decap decoupling parts between GND and the PWR islands and n_nets random-walk nets on the top
    signal layer returning in GND; n_freq log-spaced frequencies in [1 MHz, 1 GHz]."""
    rng = np.random.default_rng(seed)
    d = d_mm * 1e-3
    t = 35e-6
    side = (n - 1) * d
    length = 0.6 * n * d
    cx, cy = side * rng.uniform(0.4, 0.6), side * rng.uniform(0.4, 0.6)
    ang = rng.uniform(0, math.pi)
    cut = rect_polygon(cx, cy, length, 1e-3, ang)
    gnd = _full_layer("GND", 0.0, t, n, n, d, [cut] if slot else [])
    split_at = side * rng.uniform(0.35, 0.65)
    gap = np.array([[split_at - 0.5e-3, -d], [split_at + 0.5e-3, -d], [split_at + 0.5e-3, side + d],
                    [split_at - 0.5e-3, side + d]])
    pwr = _full_layer("PWR", -(0.2e-3 + t), t, n, n, d, [gap])
    pair = Pair(0, 1, EPS0 * 4.3 / 0.2e-3, 0.02)
    branches = []
    while len(branches) < n_decap:
        i, j = int(rng.integers(4, n - 4)), int(rng.integers(4, n - 4))
        if gnd.node[i, j] and pwr.node[i, j]:
            branches.append(BranchSpec((0, i, j), (1, i, j), 0.02, 0.5e-9, 100e-9, "part"))
    z_face, z_sig = 0.5 * t, 0.15e-3 + t
    u = np.array([math.cos(ang), math.sin(ang)])
    v = np.array([-u[1], u[0]])
    margin = max(4, n // 32)
    nets = []
    for _ in range(n_nets):
        for _ in range(1000):
            s = np.array([cx, cy]) + rng.uniform(-0.35, 0.35) * length * u - rng.uniform(0.15, 0.4) * side * v
            e = np.array([cx, cy]) + rng.uniform(-0.35, 0.35) * length * u + rng.uniform(0.15, 0.4) * side * v
            m = np.array([cx, cy]) + rng.uniform(-0.3, 0.3) * length * u
            cs, ce, cm = (np.round(p / d).astype(int) for p in (s, e, m))
            ok = all(margin <= c[0] < n - margin and margin <= c[1] < n - margin for c in (cs, ce, cm))
            if ok and gnd.node[cs[0], cs[1]] and gnd.node[ce[0], ce[1]]:
                break
        cells = _manhattan_walk(rng, cs, cm, ce, int(rng.integers(20, 61)), margin, n - 1 - margin, n - 1 - margin)
        pts = [(c[0] * d, c[1] * d) for c in cells]
        nets.append(Net(_segments(pts, z_sig, z_face, 0.15e-3), (0, int(cs[0]), int(cs[1])),
                        (0, int(ce[0]), int(ce[1]))))
    freqs = np.logspace(6, 9, n_freq)
    return Board("what_if_base", d, n, n, [gnd, pwr], [pair], branches, nets, freqs, precond="sheet", tol=1e-5,
                 restart=50)


def what_if_branches(board: Board, seed: int, n_via: int = 2, n_part: int = 1) -> list:
    """A what-if edit's added branches (the serving workload's "add 1-4 vias" / "move a decoupling part"):
    n_via stitching vias and n_part decoupling parts (ESR 20 mohm, ESL 0.5 nH, 100 nF) between two sheets at
    seeded positions where both sheets have copper and the two nodes already lie on one connected piece
    (through the plane pair or other branches), so the base's reference nodes stay."""
    from . import layout
    rng = np.random.default_rng(seed)
    t, _ = layout.topology([l.node for l in board.layers], [l.xb for l in board.layers],
                           [l.yb for l in board.layers], board.d,
                           [(p.upper, p.lower, p.c_per_area, p.tan_delta) for p in board.pairs],
                           [(b.a, b.b) for b in board.branches])
    S = len(board.layers)
    out, taken = [], {(b.a, b.b) for b in board.branches}
    for n in range(200 * (n_via + n_part)):
        if len(out) == n_via + n_part:
            break
        k0 = int(rng.integers(0, S - 1))
        k1 = int(rng.integers(k0 + 1, S))
        i, j = int(rng.integers(1, board.nx - 1)), int(rng.integers(1, board.ny - 1))
        a, b = (k0, i, j), (k1, i, j)
        na, nb = int(t.nid[a]), int(t.nid[b])
        if na < 0 or nb < 0 or t.full_label[na] != t.full_label[nb] or (a, b) in taken:
            continue
        taken.add((a, b))
        length = abs(board.layers[k0].z - board.layers[k1].z)
        if len(out) < n_via:
            out.append(BranchSpec(a, b, length / (SIGMA_CU * math.pi * 2 * 1.5e-4 * 25e-6), 2e-10 * length / 1e-3,
                                  0.0, "via", 1.5e-4))
        else:
            out.append(BranchSpec(a, b, 0.02, 0.5e-9, 100e-9, "part"))
    return out


WORKLOADS = {"plain_plane": plain_plane, "slotted_pair": slotted_pair, "small_pair": small_pair,
             "small_stack3": small_stack3, "six_sheet": six_sheet, "necked_pair": necked_pair,
             "faces_stack3": faces_stack3, "necked_faces": necked_faces}

# the analytic known-answer boards (the reference's tests/test_solver.py:19-88 and tests/test_plane_pair.py:19-81)
KNOWN_BOARDS = {
    "microstrip": lambda: microstrip(f=(1e3, 1e8)),
    "microstrip_slot6": lambda: microstrip(slot=6.0),
    "microstrip_slot12": lambda: microstrip(slot=12.0),
    "microstrip_edge_split": lambda: microstrip(edge_split=True),
    "plane_pair_line20": lambda: plane_pair_line(20.0),
    "plane_pair_line40": lambda: plane_pair_line(40.0),
}
