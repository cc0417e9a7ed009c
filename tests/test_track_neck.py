"""A neck in a track against an independent sheet solve (the reference's TW-4, tests/test_track_width.py:159-185):
a 30 mm, 0.4 mm track between two 1 mm pads with a 0.1 mm neck, 2 or 20 mm long, drawn as the reference draws it
(the union of round-capped segments, 8 segments a quarter circle, and the pads), rasterised with exact widths
(raster.build_layer, 0.25 mm pitch, sub-grid 2) and solved at DC by the oracle.  What the neck adds to the
resistance (the track without it subtracted: the pads cancel) is held to a finite-volume sheet solve of the same
copper on 0.01 mm cells (cells conducting in proportion to their copper, faces the harmonic mean, the pads held at
1 V and 0 V), written here without the solver's code: within a quarter square per end, 4 % of the 2 mm neck and
0.5 % of the 20 mm one.  CPU only."""
import math

import numpy as np
import pytest
import scipy.sparse as sp
from scipy.sparse.linalg import spsolve

from groundtruth_gb300 import raster, stack as gs, synth
from test_oracle_golden import oracle_routes, oracle_stack

SIGMA, T = 5.8e7, 35e-6
Y, X0, X1 = 10.0, 6.0, 36.0


def neck_copper(neck_len: float, neck_w: float = 0.1, wide: float = 0.4, quad: int = 8) -> np.ndarray:
    """The outline of the pads and the track (mm): a wide segment's round cap, a polygon of `quad` segments a
    quarter circle, runs into the neck until it meets the neck's edge."""
    xm0, xm1 = X0 + (X1 - X0 - neck_len) / 2, X0 + (X1 - X0 + neck_len) / 2
    big, small = wide / 2, neck_w / 2
    up = [(X0 - 0.5, Y + 0.5), (X0 + 0.5, Y + 0.5), (X0 + 0.5, Y + big)]
    if neck_len > 0:
        step = math.pi / 2 / quad
        arc = [(xm0 + big * math.cos(math.pi / 2 - a * step), Y + big * math.sin(math.pi / 2 - a * step))
               for a in range(quad + 1)]
        cap = []
        for (ax, ay), (bx, by) in zip(arc[:-1], arc[1:]):
            cap.append((ax, ay))
            if by < Y + small <= ay:
                s = (ay - (Y + small)) / (ay - by)
                cap.append((ax + s * (bx - ax), Y + small))
                break
        up += cap + [(xm0 + xm1 - px, py) for px, py in reversed(cap)]
    up += [(X1 - 0.5, Y + big), (X1 - 0.5, Y + 0.5), (X1 + 0.5, Y + 0.5)]
    return np.array([(px, 2 * Y - py) for px, py in up] + list(reversed(up)))


def sheet_resistance(outline: np.ndarray, h: float) -> float:
    """The copper's resistance between the two pads by a finite-volume sheet solve on cells of h mm."""
    pa, pb = raster.ring_edges(outline)
    lo, hi = outline.min(axis=0), outline.max(axis=0)
    xl, yl = lo[0] - h, lo[1] - h
    wi, wj = int(math.ceil((hi[0] - lo[0]) / h)) + 2, int(math.ceil((hi[1] - lo[1]) / h)) + 2
    right = raster.line_cover(pa[:, 0], pa[:, 1], pb[:, 0], pb[:, 1], xl + h, h, wi, yl + h / 2, h, wj)
    c = raster.cell_areas(pa, pb, xl, yl, h, wi, wj, right) / (h * h)
    X, Y_ = np.meshgrid(xl + (np.arange(wi) + 0.5) * h, yl + (np.arange(wj) + 0.5) * h, indexing="ij")
    held = [(np.abs(X - x) < 0.5) & (np.abs(Y_ - Y) < 0.5) for x in (X0, X1)]        # the pads: 1 V, 0 V
    free = (c > 1e-9) & ~held[0] & ~held[1]
    idx = -np.ones((wi, wj), np.int64)
    n = int(free.sum())
    idx[free] = np.arange(n)
    rows, cols, vals, diag, rhs = [], [], [], np.zeros(n), np.zeros(n)
    faces = []
    for di, dj in ((1, 0), (0, 1)):
        a, b = (slice(0, wi - di), slice(0, wj - dj)), (slice(di, wi), slice(dj, wj))
        g = np.where((c[a] > 0) & (c[b] > 0), SIGMA * T * 2 * c[a] * c[b] / np.maximum(c[a] + c[b], 1e-30), 0.0)
        faces.append((a, b, g))
        ia, ib = idx[a], idx[b]
        m = (ia >= 0) & (ib >= 0) & (g > 0)
        rows += [ia[m], ib[m]]
        cols += [ib[m], ia[m]]
        vals += [-g[m], -g[m]]
        np.add.at(diag, ia[m], g[m])
        np.add.at(diag, ib[m], g[m])
        for pad, volts in zip(held, (1.0, 0.0)):
            for i_free, other in ((ia, b), (ib, a)):
                m = (i_free >= 0) & pad[other] & (g > 0)
                np.add.at(diag, i_free[m], g[m])
                np.add.at(rhs, i_free[m], g[m] * volts)
    A = sp.coo_matrix((np.concatenate(vals + [diag]), (np.concatenate(rows + [np.arange(n)]),
                                                      np.concatenate(cols + [np.arange(n)]))), shape=(n, n)).tocsr()
    V = np.zeros((wi, wj))
    V[free] = spsolve(A, rhs)
    V[held[0]] = 1.0
    current = sum(float(np.sum(np.where(held[0][a] & ~held[0][b], g * (1.0 - V[b]), 0.0)
                               + np.where(held[0][b] & ~held[0][a], g * (1.0 - V[a]), 0.0))) for a, b, g in faces)
    return 1.0 / current


def peec_resistance(neck_len: float, d: float = 0.25, sub: int = 2) -> float:
    """The same copper through raster.build_layer (the track's centreline forced, as the reference's tracks are)
    and the oracle's DC solve between the pads' centre nodes."""
    xm0, xm1 = X0 + (X1 - X0 - neck_len) / 2, X0 + (X1 - X0 + neck_len) / 2
    runs = [((X0, Y), (xm0, Y), 0.4), ((xm0, Y), (xm1, Y), 0.1), ((xm1, Y), (X1, Y), 0.4)] if neck_len else \
        [((X0, Y), (X1, Y), 0.4)]
    g = raster.build_layer({"PWR": [(neck_copper(neck_len), [])]}, (0.0, 0.0, 42.0, 20.0), d,
                           lines={"PWR": [(np.array([a, b]), w) for a, b, w in runs]}, sub=sub)
    grid = gs.Grid(0.0, 0.0, d, g.nx, g.ny, g.node, g.xb, g.yb)
    ends = [(0, *grid.nearest_node(x, Y)) for x in (X0, X1)]
    layer = synth.Layer("F", 0.0, T, g.node, g.xb, g.yb, g.widths(), g.fill, g.area, g.label)
    board = synth.Board("neck", d * 1e-3, g.nx, g.ny, [layer], nets=[synth.Net(np.zeros((0, 8)), *ends)],
                        freqs=np.array([0.0]), tol=1e-12)
    return oracle_routes(oracle_stack(board), board)[0].solve(0.0, tol=1e-12)["Z_loop"].real


@pytest.mark.parametrize("neck_len, rel", [(2.0, 0.04), (20.0, 0.005)])
def test_a_neck_against_an_independent_sheet_solve(neck_len, rel):
    ref = {h: sheet_resistance(neck_copper(neck_len), h) - sheet_resistance(neck_copper(0.0), h) for h in (0.02, 0.01)}
    assert ref[0.01] == pytest.approx(ref[0.02], rel=0.01)                  # the sheet solve is converged
    added = peec_resistance(neck_len) - peec_resistance(0.0)
    square = 1 / (SIGMA * T)
    assert abs(added - ref[0.01]) <= 2 * 0.25 * square                    # a quarter square per end
    assert added == pytest.approx(ref[0.01], rel=rel)
