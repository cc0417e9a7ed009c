"""Golden vectors of the exact-copper raster's arithmetic (peec.py:482-705) from GroundTruth itself.

    python tests/golden/make_raster_golden.py --reference /path/to/GroundTruth

Seeded polygons (as edge lists, groundtruth_gb300.raster.ring_edges) and arrays go through the reference's
_line_cover, _cell_areas, _strip_widths, _adopt and _series_factor, and seeded layers and polylines through its
track walk _rasterise_lines; inputs and outputs are stored in raster_functions.npz (shapely is stubbed: none of
these functions calls it)."""
from __future__ import annotations

import argparse
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from groundtruth_gb300 import raster  # noqa: E402


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
    np.savez_compressed(HERE / "raster_functions.npz", **out)


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
