"""Golden vectors of the raster (peec.py:329-449, 482-849, 893-983) from GroundTruth itself.

    python tests/golden/make_raster_golden.py --reference /path/to/GroundTruth

Seeded polygons (as edge lists, groundtruth_gb300.raster.ring_edges) and arrays go through the reference's
_line_cover, _cell_areas, _strip_widths, _adopt and _series_factor, and seeded layers and polylines through its
track walk _rasterise_lines, and three nets' copper through its sub-grid rasteriser _coarse_from_fine and its
exact-copper pass _exact_copper; inputs and outputs are stored in raster_functions.npz.  shapely is stubbed: the
first functions do not call it; for the last two its point test is synth.copper_at and a net's edges and bounds
are given as ring_edges and the outline's extent, so the vectors pin everything of those two but the point test
itself.  build_grid itself (a layer at sub = 1, 4 and 3 with seeds and tracks) runs on the same stubs, its
pieces given and its thermal heat points left out."""
from __future__ import annotations

import argparse
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from groundtruth_gb300 import raster, synth  # noqa: E402


def polygons(rng):
    """A star-shaped outline with two rectangular holes, mm."""
    ang = np.sort(rng.uniform(0, 2 * np.pi, 14))
    rad = rng.uniform(3.0, 6.0, 14)
    outline = np.stack([8 + rad * np.cos(ang), 8 + rad * np.sin(ang)], 1)
    holes = [np.array([[6.1, 6.3], [7.4, 6.3], [7.4, 9.05], [6.1, 9.05]]),
             np.array([[9.2, 7.7], [10.15, 7.7], [10.15, 8.6], [9.2, 8.6]])]
    return outline, holes


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    args = ap.parse_args()
    sys.modules.setdefault("shapely", types.ModuleType("shapely"))
    sys.path.insert(0, str(Path(args.reference) / "src"))
    from groundtruth.solver import peec
    rng = np.random.default_rng(41)
    out = {}
    outline, holes = polygons(rng)
    pa, pb = raster.ring_edges(outline, holes)
    out.update(pa=pa, pb=pb)
    d, xl, yl, wi, wj = 0.35, 1.3, 1.1, 40, 42
    # covered length of each cell's right border (vertical lines x = xl + (i+1) d) and of the top borders
    right = peec._line_cover(pa[:, 0], pa[:, 1], pb[:, 0], pb[:, 1], xl + d, d, wi, yl + d / 2, d, wj)
    top = peec._line_cover(pa[:, 1], pa[:, 0], pb[:, 1], pb[:, 0], yl + d, d, wj, xl + d / 2, d, wi)
    out.update(right=right, top=top, areas=peec._cell_areas(pa, pb, xl, yl, d, wi, wj, right))
    exists = rng.random((30, 20)) < 0.8
    cross = np.where(rng.random((30, 20)) < 0.7, rng.uniform(0, 1.2, (30, 20)), 0.0)
    offset = rng.uniform(-0.6, 0.6, (30, 20))
    forced = np.where(rng.random((30, 20)) < 0.2, rng.uniform(0, 0.5, (30, 20)), 0.0)
    exact = np.where(rng.random((30, 20)) < 0.5, rng.uniform(0, 3.5, (30, 20)), 0.0)
    w0, o0 = peec._strip_widths(exists, cross, offset, forced, 0.25)
    w1, o1 = peec._strip_widths(exists, cross, offset, forced, 0.25, exact)
    out.update(sw_exists=exists, sw_cross=cross, sw_offset=offset, sw_forced=forced, sw_exact=exact,
               sw_w0=w0, sw_o0=o0, sw_w1=w1, sw_o1=o1)
    cov = np.where(rng.random((25, 23)) < 0.6, rng.uniform(0, 1, (25, 23)), 0.0)
    has = rng.random((25, 23)) < 0.5
    steps = [(0, 1), (0, -1), (1, 0), (-1, 0)]
    out.update(ad_cov=cov, ad_has=has, ad_1=peec._adopt(cov, has, steps), ad_3=peec._adopt(cov, has, steps, 3))
    has_s = np.zeros((28, 26), bool)
    has_s[3:6, 4:20] = True           # a narrow band along axis 1
    has_s[12, :] = True               # a single long run
    has_s[18:26, 7:9] = True          # a wider band
    has_s[20, 15:18] = True
    face = rng.uniform(0.2, 1.0, (28, 26))
    samples = [face * rng.uniform(0.5, 1.5, (28, 26)) for _ in range(3)]
    for ax in (0, 1):
        out[f"sf_{ax}"] = peec._series_factor(face, samples, has_s, ax)
    out.update(sf_face=face, sf_samples=np.stack(samples), sf_has=has_s)
    out.update(track_cases(peec, rng))
    out.update(copper_cases(peec, rng))
    out.update(layer_cases(peec, rng))
    np.savez_compressed(HERE / "raster_functions.npz", **out)


class _Net:
    """A net's copper for build_grid without shapely: its pieces (each a _Copper), the union's bounds and edges."""

    def __init__(self, pieces):
        self.pieces = [_Copper(o, h) for o, h in pieces]
        lo = np.min([p.outline.min(axis=0) for p in self.pieces], axis=0)
        hi = np.max([p.outline.max(axis=0) for p in self.pieces], axis=0)
        self.bounds = (float(lo[0]), float(lo[1]), float(hi[0]), float(hi[1]))
        self.is_empty = False
        self.pa = np.concatenate([p.pa for p in self.pieces])
        self.pb = np.concatenate([p.pb for p in self.pieces])
        self.outline = None


def layer_nets(rng) -> dict:
    """{net: pieces}: a pour with holes, a track, and a supply of two separate pads."""
    pour, track, pad = copper_nets(rng)
    pad2 = (np.array([[17.2, 3.3], [18.9, 3.3], [18.9, 4.6], [17.2, 4.6]]), [])
    return {"GND": [pour], "SIG": [track], "VCC": [pad, pad2]}


POINTS = [(2.0, 2.0), (10.3, 9.1), (17.9, 4.1), (12.0, 17.6), (30.0, 5.0), (0.0, 24.0)]


def layer_cases(peec, rng) -> dict:
    """build_grid of the reference on one layer at sub = 1, 4 and 3, with seeds and tracks (shapely stubbed as in
    copper_cases: the point test synth.copper_at, covers with its border; the thermal heat points left out)."""
    stub = sys.modules["shapely"]

    def contains(g, X, Y):
        polys = g.pieces if isinstance(g, _Net) else [g]
        out = np.zeros(np.shape(X), bool)
        for p in polys:
            out |= synth.copper_at(X, Y, p.outline, p.holes)
        return out

    class _Tree:
        def __init__(self, items):
            self.n = len(items)

        def query(self, point):
            return np.arange(self.n)

    def covers(self, pt):
        return bool(raster._covers(np.array([pt[0]]), np.array([pt[1]]), (self.outline, self.holes))[0])
    stub.contains_xy = contains
    stub.STRtree = _Tree
    stub.Point = lambda x, y: (x, y)
    _Copper.covers = covers
    peec._pieces = lambda g: g.pieces
    peec._heat_points = lambda geoms, label, x0, y0, d: (np.zeros(label.shape), np.zeros(label.shape))
    nets = layer_nets(rng)
    seeds = {"GND": [(4.0, 12.0), (10.1, 9.6), (2.9, 2.7)], "VCC": [(18.0, 4.0), (30.0, 30.0)], "NC": [(1.0, 1.0)]}
    lines = {"SIG": [(np.array([[5.2, 14.3], [11.0, 16.1], [19.4, 20.2]]), 0.2)],
             "GND": [(np.array([[3.0, 3.0], [3.0, 6.5], [6.0, 6.5]]), 0.25)],
             "VCC": [(np.array([[2.8, 2.6], [17.9, 3.9]]), 0.3)]}
    out = {}
    for name, piece_list in nets.items():
        for m, (o, h) in enumerate(piece_list):
            out[f"ly_{name}_{m}_outline"] = o
            for q, hole in enumerate(h):
                out[f"ly_{name}_{m}_hole{q}"] = hole
    for case, (bbox, d, sub) in {"s1": ((0.3, 0.2, 21.0, 24.5), 0.5, 1), "s4": ((0.3, 0.2, 21.0, 24.5), 0.5, 4),
                                 "s3": ((-0.4, 0.9, 20.6, 22.0), 0.7, 3)}.items():
        g = peec.build_grid({n: _Net(p) for n, p in nets.items()}, bbox, d, seeds, lines, sub)
        out.update({f"ly_{case}_node": g.node, f"ly_{case}_xb": g.xb, f"ly_{case}_yb": g.yb,
                    f"ly_{case}_label": g.label, f"ly_{case}_bridges": np.array(g.bridges, float).reshape(-1, 6)})
        # the grid's lookups: nearest copper node (any net, one net, within a distance), a node's net, extent
        near = []
        for x, y in POINTS:
            for net, dist in ((None, None), ("VCC", None), ("SIG", 1.0), ("GND", 0.3), ("NC", None)):
                n = g.nearest_node(x, y, dist, net)
                near.append((-1, -1) if n is None else n)
        out[f"ly_{case}_near"] = np.array(near, np.int64)
        out[f"ly_{case}_net_at"] = np.array([g.net_at(tuple(n)) if n[0] >= 0 else "" for n in near])
        out[f"ly_{case}_extent"] = np.array(g.extent)
        for key in ("fill", "wx", "wy", "ox", "oy", "area", "rx", "ry"):
            if getattr(g, key) is not None:
                out[f"ly_{case}_{key}"] = getattr(g, key)
    return out

class _Copper:
    """A net's copper for the reference's functions without shapely: its rings' oriented edges and bounds
    (what _ring_edges and .bounds give), and its polygon for the point test."""

    def __init__(self, outline, holes):
        self.outline, self.holes = outline, holes
        self.pa, self.pb = raster.ring_edges(outline, holes)
        lo, hi = outline.min(axis=0), outline.max(axis=0)
        self.bounds = (float(lo[0]), float(lo[1]), float(hi[0]), float(hi[1]))
        self.is_empty = False


def copper_nets(rng) -> list:
    """Three nets of a layer, mm: a star-shaped pour with two holes, a track 0.3 mm wide at 23 degrees, and a
    small pad."""
    ang = np.sort(rng.uniform(0, 2 * np.pi, 16))
    rad = rng.uniform(4.0, 7.0, 16)
    pour = (np.stack([10 + rad * np.cos(ang), 9 + rad * np.sin(ang)], 1),
            [np.array([[8.1, 8.3], [9.4, 8.3], [9.4, 11.05], [8.1, 11.05]]),
             np.array([[11.2, 7.7], [12.15, 7.7], [12.15, 8.6], [11.2, 8.6]])])
    track = (synth.rect_polygon(12.0, 17.5, 14.0, 0.3, np.radians(23.0)), [])
    pad = (np.array([[2.3, 2.2], [3.45, 2.2], [3.45, 3.1], [2.3, 3.1]]), [])
    return [pour, track, pad]


def copper_cases(peec, rng) -> dict:
    """The sub-grid rasteriser (_coarse_from_fine, s = 4) and the exact-copper pass (_exact_copper) of the
    reference on three nets; the sub-grid's point test is synth.copper_at (standing in for shapely.contains_xy)."""
    stub = sys.modules["shapely"]
    stub.prepare = lambda g: None
    stub.contains_xy = lambda g, X, Y: synth.copper_at(X, Y, g.outline, g.holes)
    peec._ring_edges = lambda g: (g.pa, g.pb)
    nets = copper_nets(rng)
    geoms = [_Copper(o, h) for o, h in nets]
    x0, y0, d, nx, ny, s = 0.4, 0.3, 0.5, 44, 46, 4
    label, cx, cy, fill, ox, oy = peec._coarse_from_fine(geoms, x0, y0, d, nx, ny, s)
    xb = (label[:-1, :] >= 0) & (label[:-1, :] == label[1:, :]) & (cx > 0)
    yb = (label[:, :-1] >= 0) & (label[:, :-1] == label[:, 1:]) & (cy > 0)
    ex_x, ex_y, area, kx, ky = peec._exact_copper(geoms, label, xb, yb, x0, y0, d)
    out = {"cu_label": label, "cu_cx": cx, "cu_cy": cy, "cu_fill": fill, "cu_ox": ox, "cu_oy": oy, "cu_xb": xb,
           "cu_yb": yb, "cu_ex_x": ex_x, "cu_ex_y": ex_y, "cu_area": area, "cu_kx": kx, "cu_ky": ky}
    for k, (o, h) in enumerate(nets):
        out[f"cu_net{k}_outline"] = o
        for m, hole in enumerate(h):
            out[f"cu_net{k}_hole{m}"] = hole
    return out

def track_cases(peec, rng) -> dict:
    """Seeded layers (free cells, net 2's cells in two pieces, other nets' cells) with polylines partly off the
    grid, through the reference's _rasterise_lines without and with pieces: inputs and every updated array."""
    out = {}
    nx, ny, d, x0, y0, k = 30, 24, 0.5, 1.0, 2.0, 2
    lines = []
    for n in range(6):
        m = int(rng.integers(2, 6))
        pts = np.stack([rng.uniform(x0 - 1.5, x0 + nx * d + 1.0, m), rng.uniform(y0 - 1.0, y0 + ny * d + 1.5, m)], 1)
        lines.append((pts, 0.0 if n == 2 else float(rng.uniform(0.1, 0.6))))
    out.update(tr_pts=np.concatenate([p for p, _ in lines]), tr_ptr=np.cumsum([0] + [len(p) for p, _ in lines]),
               tr_width=np.array([w for _, w in lines]), tr_owners=np.array([n % 2 for n in range(len(lines))]))
    for case, pieces in (("plain", False), ("pieces", True)):
        r = rng.random((nx, ny))
        label = np.where(r < 0.6, -1, np.where(r < 0.8, k, rng.integers(0, 2, (nx, ny)) * 2 - 1 + (r > 0.9) * 4))
        label = np.where(label == k, k, np.where(label < 0, -1, label))
        part = np.where(label == k, rng.integers(0, 2, (nx, ny)), -1) if pieces else None
        seeded = np.zeros((nx, ny), bool)
        fx, fy = np.zeros((nx - 1, ny)), np.zeros((nx, ny - 1))
        out.update({f"tr_{case}_label0": label.copy()})
        if pieces:
            out[f"tr_{case}_part0"] = part.copy()
        br = peec._rasterise_lines(k, lines, x0, y0, d, label, seeded, fx, fy, part,
                                   [n % 2 for n in range(len(lines))] if pieces else None)
        out.update({f"tr_{case}_label": label, f"tr_{case}_seeded": seeded, f"tr_{case}_fx": fx,
                    f"tr_{case}_fy": fy, f"tr_{case}_bridges": np.array(br, float).reshape(-1, 6)})
        if pieces:
            out[f"tr_{case}_part"] = part
    return out


if __name__ == "__main__":
    main()
