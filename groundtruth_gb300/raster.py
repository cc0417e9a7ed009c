"""Copper polygons and tracks onto the solver's grid (GroundTruth: build_grid and its helpers, peec.py:329-983), the
parts that need no polygon library.

* The exact-copper arithmetic (peec.py:482-771): how much copper crosses each cell border along scanlines
  (line_cover), each cell's copper area by Green's theorem (cell_areas), a strip's width and centre from those
  (strip_widths), copper of a border without a strip of its net moved to the nearest strip that has one (adopt),
  the series factor of a narrow run whose width changes along its length (series_factor), and the pass over a
  net's copper that measures them (exact_copper).
* The sub-grid rasteriser (coarse_from_fine, peec.py:774-849), the walk that claims tracks' cells and strips
  (rasterise_tracks, peec.py:893-983), a net's polygons grouped into pieces (pieces, peec.py:852-873) and the
  layer rasteriser around them (build_layer, peec.py:329-449).

Polygons are (outline, holes) vertex arrays, or their edges (outlines counter-clockwise, holes clockwise:
ring_edges), in the same length unit as the pitch."""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

BAND_STRIPS = 4      # peec.py:108: a narrow conductor is a band of at most this many side-by-side strips ...
ADOPT_FACES = 3      # peec.py:110: ... with no other strip of its net within 2 x this many faces along the border


def ring_edges(outline: np.ndarray, holes=()) -> tuple:
    """(start, end) points of a polygon's edges with the copper on their left: the outline counter-clockwise,
    each hole clockwise (what shapely's orient_polygons gives the reference, peec.py:516-531)."""
    def oriented(ring, ccw):
        ring = np.asarray(ring, float)
        area = 0.5 * np.sum(ring[:, 0] * np.roll(ring[:, 1], -1) - np.roll(ring[:, 0], -1) * ring[:, 1])
        return ring if (area > 0) == ccw else ring[::-1]
    a, b = [], []
    for ring, ccw in [(outline, True)] + [(h, False) for h in holes]:
        r = oriented(ring, ccw)
        a.append(r)
        b.append(np.roll(r, -1, axis=0))
    return np.concatenate(a), np.concatenate(b)


def _ragged(start, count) -> tuple:
    """The members of integer ranges [start_i, start_i + count_i): (owner i, value) pairs, owners ascending."""
    count = np.maximum(np.asarray(count, np.int64), 0)
    owner = np.repeat(np.arange(len(count)), count)
    base = np.cumsum(count) - count
    return owner, np.asarray(start, np.int64)[owner] + (np.arange(len(owner)) - base[owner])


def line_cover(ua, va, ub, vb, u0: float, du: float, n_lines: int, v0: float, d: float, n_cells: int) -> np.ndarray:
    """(n_lines, n_cells): on each line u = u0 + m du, the length of each cell interval
    [v0 + (c - 1/2) d, v0 + (c + 1/2) d] that lies inside the polygons whose edges run (ua, va) -> (ub, vb)
    (peec.py:533-580).  An edge meets the lines whose u lies in [min, max) of its ends' u (a vertex on a line
    counts once, an edge along a line not at all); a line's crossings, sorted along it, alternate entering and
    leaving the copper, and a line meeting an odd number of them is left empty.  With crossings c_1 < c_2 < ...
    the covered length below v is sum_k (-1)^(k+1) (v - c_k)_+, so each crossing adds +-d to every cell from
    its own on, less +-(c_k - its cell's lower end) in its own cell: a running sum along the line (a crossing
    on a cell's lower end adds exactly nothing to that cell)."""
    out = np.zeros((n_lines, n_cells))
    ua, va, ub, vb = (np.asarray(a, float).ravel() for a in (ua, va, ub, vb))
    if not len(ua) or n_lines <= 0 or n_cells <= 0:
        return out
    lo = np.clip(np.ceil((np.minimum(ua, ub) - u0) / du), 0, n_lines).astype(np.int64)
    hi = np.clip(np.ceil((np.maximum(ua, ub) - u0) / du), 0, n_lines).astype(np.int64)
    e, line = _ragged(lo, hi - lo)
    if not len(e):
        return out
    t = (u0 + line * du - ua[e]) / (ub[e] - ua[e])
    v = va[e] + t * (vb[e] - va[e])
    order = np.lexsort((v, line))
    line, v = line[order], v[order]
    first = np.searchsorted(line, line)
    rank = np.arange(len(line)) - first
    count = np.bincount(line, minlength=n_lines)
    keep = count[line] % 2 == 0
    line, v, sign = line[keep], v[keep], np.where(rank[keep] % 2 == 0, 1.0, -1.0)
    span = n_cells * d
    x = np.clip(v - (v0 - 0.5 * d), 0.0, span)
    cell = np.minimum((x / d).astype(np.int64), n_cells - 1)
    steps = np.bincount(line * n_cells + cell, sign * d, n_lines * n_cells).reshape(n_lines, n_cells)
    out += np.cumsum(steps, axis=1)
    out.reshape(-1)[:] -= np.bincount(line * n_cells + cell, sign * (x - cell * d), n_lines * n_cells)
    return out


def cell_areas(pa, pb, xl: float, yl: float, d: float, wi: int, wj: int, right: np.ndarray) -> np.ndarray:
    """(wi, wj): the copper area of each cell [xl + i d, xl + (i+1) d] x [yl + j d, yl + (j+1) d] inside the
    polygons with oriented edges pa -> pb, copper on their left, `right` the covered length of each cell's right
    border (line_cover's convention; the areas of peec.py:583-622).  Green's theorem over the boundary of
    copper-and-cell, area = closed int (x - x_i) dy: the cell's right border adds d times its covered length, its
    left border nothing, and each polygon edge adds (its mean x - x_i) dy over every stretch of it that lies in
    the cell.  An edge is cut into its stretches per column (a vertical edge on a border line belongs to the
    column on its right, where it adds nothing) and each stretch per row."""
    out = d * np.asarray(right, float)
    pa, pb = np.asarray(pa, float).reshape(-1, 2), np.asarray(pb, float).reshape(-1, 2)
    if not len(pa):
        return out
    xa, ya, xb, yb = pa[:, 0], pa[:, 1], pb[:, 0], pb[:, 1]
    keep = ya != yb                                       # edges along a row add no dy
    xa, ya, xb, yb = xa[keep], ya[keep], xb[keep], yb[keep]
    vertical = xa == xb
    c0 = np.floor((np.minimum(xa, xb) - xl) / d).astype(np.int64)
    c1 = np.floor((np.maximum(xa, xb) - xl) / d).astype(np.int64)
    lo, hi = np.clip(c0, 0, wi - 1), np.clip(c1, 0, wi - 1)
    e, col = _ragged(lo, np.where((c1 >= 0) & (c0 < wi), hi - lo + 1, 0))
    # each stretch's x range and the y at its ends
    left = xl + col * d
    xs = np.maximum(np.minimum(xa[e], xb[e]), left)
    xe = np.minimum(np.maximum(xa[e], xb[e]), left + d)
    vert = vertical[e]
    use = vert | (xe > xs)
    e, col, xs, xe, vert, left = e[use], col[use], xs[use], xe[use], vert[use], left[use]
    with np.errstate(divide="ignore", invalid="ignore"):
        slope = np.where(vert, 0.0, (yb[e] - ya[e]) / np.where(vert, 1.0, xb[e] - xa[e]))
    ys = np.where(vert, ya[e], ya[e] + (xs - xa[e]) * slope)
    ye = np.where(vert, yb[e], ya[e] + (xe - xa[e]) * slope)
    # dy's sign is the edge's direction; the stretch runs from its lower end (x at it xlo) to its upper one
    up = yb[e] > ya[e]
    ylo, yhi = np.minimum(ys, ye), np.maximum(ys, ye)
    xlo = np.where(ys <= ye, xs, xe)
    xhi = np.where(ys <= ye, xe, xs)
    r0 = np.floor((ylo - yl) / d).astype(np.int64)
    r1 = np.floor((yhi - yl) / d).astype(np.int64)
    rlo, rhi = np.clip(r0, 0, wj - 1), np.clip(r1, 0, wj - 1)
    k, row = _ragged(rlo, np.where((r1 >= 0) & (r0 < wj), rhi - rlo + 1, 0))
    bottom = yl + row * d
    y0, y1 = np.maximum(ylo[k], bottom), np.minimum(yhi[k], bottom + d)
    ok = y1 > y0
    k, row, y0, y1 = k[ok], row[ok], y0[ok], y1[ok]
    xm = xlo[k] + (0.5 * (y0 + y1) - ylo[k]) / (yhi[k] - ylo[k]) * (xhi[k] - xlo[k])
    np.add.at(out, (col[k], row), np.where(up[k], 1.0, -1.0) * (xm - left[k]) * (y1 - y0))
    return out


def strip_widths(exists, cross, offset, forced, d: float, exact=None) -> tuple:
    """Each strip's copper width as a fraction of the pitch and its centre's offset across the strip
    (peec.py:482-513): the exact covered border where measured (at most 3 pitches: a strip carries the sliver
    beside it too), else the share of its border the sub-grid saw copper cross, at least a forced track's own
    width, 1 where neither; the centre kept inside the cell; 0 where no strip exists."""
    exists = np.asarray(exists, bool)
    cross, offset, forced = (np.asarray(a, float) for a in (cross, offset, forced))
    # the sub-grid's estimate: the crossed share of the border, raised to a claiming track's own width
    track = np.where(forced > 0, np.minimum(forced / d, 1.0), 0.0)
    seen = np.maximum(cross, track)
    picks = [seen > 0]
    vals = [np.minimum(seen, 1.0)]
    if exact is not None:
        exact = np.asarray(exact, float)
        picks.insert(0, exact > 0)
        vals.insert(0, np.minimum(exact, 3.0))
    w = np.select(picks, vals, default=1.0)
    room = np.maximum(0.5 * (1.0 - w), 0.0)
    o = np.clip(np.where(cross > 0, offset, 0.0), -room, room)
    return np.where(exists, w, 0.0), np.where(exists, o, 0.0)


def adopt(cov, has, steps, reach: int = 1) -> np.ndarray:
    """`cov` where `has`, plus the values where nothing of the net exists moved to the nearest place that has one
    along the offsets `steps` within `reach` steps (of two at one distance, the one with more copper of its own);
    values with none within reach are dropped (peec.py:625-656)."""
    cov, has = np.asarray(cov, float), np.asarray(has, bool)
    ni, nj = cov.shape
    out = np.where(has, cov, 0.0)
    own = out.copy()
    stray = np.where(has, 0.0, cov)
    ii, jj = np.nonzero(stray > 0)
    amount = stray[ii, jj]
    for k in range(1, reach + 1):
        if not len(ii):
            break
        # the candidates at distance k along each step: their own copper where the net is there, else -1
        cand = np.full((len(steps), len(ii)), -1.0)
        ti = np.empty((len(steps), len(ii)), np.int64)
        tj = np.empty_like(ti)
        for q, (di, dj) in enumerate(steps):
            ti[q], tj[q] = ii + k * di, jj + k * dj
            on = (ti[q] >= 0) & (ti[q] < ni) & (tj[q] >= 0) & (tj[q] < nj)
            hit = np.zeros(len(ii), bool)
            hit[on] = has[ti[q][on], tj[q][on]]
            cand[q, hit] = own[ti[q][hit], tj[q][hit]]
        best = np.argmax(cand, axis=0)                    # the first of equals: steps' order breaks ties
        found = cand[best, np.arange(len(ii))] >= 0
        np.add.at(out, (ti[best, np.arange(len(ii))][found], tj[best, np.arange(len(ii))][found]), amount[found])
        ii, jj, amount = ii[~found], jj[~found], amount[~found]
    return out


def series_factor(face, samples: list, has, axis: int) -> np.ndarray:
    """Per strip, the conductance change of its band (a run of side-by-side strips in one column, `axis` 1: x
    strips by rows, 0: y strips by columns) when the copper's width is taken along the strips' length instead of at
    the border: the harmonic mean of the band's total width at the sample lines over its total at the border, for a
    lone narrow band only (at most BAND_STRIPS strips, no other strip of the net within 2 ADOPT_FACES along the
    border, copper at every sample line); 1 otherwise (peec.py:659-705)."""
    has = np.asarray(has, bool)
    if not has.any():
        return np.ones(has.shape)
    along = (lambda a: np.asarray(a, float)) if axis == 1 else (lambda a: np.asarray(a, float).T)
    h = has if axis == 1 else has.T
    n0, n1 = h.shape
    # the bands: runs of strips along each row; +1 where one begins, -1 just past its end
    edge = np.diff(np.pad(h.astype(np.int8), ((0, 0), (1, 1))), axis=1)
    row, beg = np.nonzero(edge == 1)
    _, end = np.nonzero(edge == -1)
    size = end - beg
    wide = 2 * ADOPT_FACES
    same_prev = np.r_[False, row[1:] == row[:-1]]
    same_next = np.r_[row[1:] == row[:-1], False]
    gap_before = np.where(same_prev, beg - np.r_[0, end[:-1]], wide + 1)
    gap_after = np.where(same_next, np.r_[beg[1:], 0] - end, wide + 1)
    lone = (size <= BAND_STRIPS) & (gap_before > wide) & (gap_after > wide)
    heads = np.cumsum(size) - size

    def band_sum(a):
        return np.add.reduceat(along(a)[h], heads)
    total = band_sum(face)
    widths = np.stack([band_sum(smp) for smp in samples])          # (samples, bands)
    seen = np.all(widths > 0, axis=0)
    harmonic = len(samples) / np.maximum(np.sum(1.0 / np.maximum(widths, 1e-300), axis=0), 1e-300)
    factor = np.where(lone & seen & (total > 0), harmonic / np.maximum(total, 1e-300), 1.0)
    out = np.ones(h.shape)
    out[h] = np.repeat(factor, size)
    return out if axis == 1 else out.T


TRACK_SAMPLE = 0.4   # peec.py:939: a centreline is sampled every 0.4 pitch, so that no cell is skipped


def _nearest_cells(u: float, v: float) -> list:
    """The four cells around grid point (u, v) (pitch units), nearest first; ties keep the order (i0, j0),
    (i0, j0 + 1), (i0 + 1, j0), (i0 + 1, j0 + 1)."""
    i0, j0 = math.floor(u), math.floor(v)
    four = [(i0, j0), (i0, j0 + 1), (i0 + 1, j0), (i0 + 1, j0 + 1)]
    return sorted(four, key=lambda c: (c[0] - u) ** 2 + (c[1] - v) ** 2)


def _l_path(a: tuple, b: tuple, blocked) -> list:
    """The 4-connected cells from a (excluded) to b (included) along an L: along i first or along j first,
    whichever crosses fewer blocked cells (along i on a tie)."""
    di, dj = b[0] - a[0], b[1] - a[1]
    si, sj = (di > 0) - (di < 0), (dj > 0) - (dj < 0)
    leg_i = [(a[0] + si * n, a[1]) for n in range(1, abs(di) + 1)]
    leg_j = [(a[0], a[1] + sj * n) for n in range(1, abs(dj) + 1)]
    i_first = leg_i + [(b[0], c[1]) for c in leg_j]
    j_first = leg_j + [(c[0], b[1]) for c in leg_i]
    cost = [sum(1 for c in p if blocked(c)) for p in (i_first, j_first)]
    return i_first if cost[0] <= cost[1] else j_first


def rasterise_tracks(k: int, polylines, x0: float, y0: float, d: float, label: np.ndarray, seeded: np.ndarray,
                     forced_x: np.ndarray, forced_y: np.ndarray, part: Optional[np.ndarray] = None,
                     owners: Optional[list] = None) -> list:
    """Tracks (polylines [(points (p, 2), width)], in the unit of x0, y0 and d) claimed on a layer's cell grid
    for net k (GroundTruth's _rasterise_lines, peec.py:893-983); label (cells' nets, -1 free), seeded, forced_x /
    forced_y (the widest claiming track's width per strip) and part are updated in place.

    Each centreline is walked one sample every TRACK_SAMPLE pitch: at a sample the walk takes, of the four
    cells around it (nearest first), the first that is already the track's own (net k's, and of the track's
    piece of copper when `part` / `owners` give pieces), else the first that may be claimed (free or own), else
    the nearest; a cell that differs from the last is reached along the L path through fewer cells that may not
    be claimed.  Then, in walk order, free cells on the grid are claimed (and seeded); consecutive own cells one
    step apart force their strip's width; an own cell reached across cells the track could not claim starts a
    bridge from the last own cell: returned as (i0, j0, i1, j1, length along the track (at least d), width), a
    lumped branch for the caller."""
    nx, ny = label.shape
    bridges = []
    for n_line, (pts, width) in enumerate(polylines):
        piece = owners[n_line] if owners is not None else None

        def on_grid(c):
            return 0 <= c[0] < nx and 0 <= c[1] < ny

        def own(c):
            return on_grid(c) and label[c] == k and (part is None or piece is None or part[c] == piece)

        def claimable(c):
            return on_grid(c) and (label[c] == -1 or own(c))

        walk = []                                          # (i, j, distance along the centreline)
        start = 0.0
        for (ax, ay), (bx, by) in zip(pts, pts[1:]):
            seg = math.hypot(bx - ax, by - ay)
            for t in np.linspace(0.0, 1.0, max(int(math.ceil(seg / (TRACK_SAMPLE * d))), 1) + 1):
                near = _nearest_cells((ax + t * (bx - ax) - x0) / d, (ay + t * (by - ay) - y0) / d)
                cell = next((c for c in near if own(c)), None) or next((c for c in near if claimable(c)), near[0])
                s = start + t * seg
                if not walk:
                    walk.append((cell[0], cell[1], s))
                elif walk[-1][:2] != cell:
                    walk.extend((c[0], c[1], s) for c in _l_path(walk[-1][:2], cell, lambda c: not claimable(c)))
            start += seg
        prev, last = None, None
        for i, j, s in walk:
            if not on_grid((i, j)):
                prev = last = None
                continue
            if label[i, j] < 0:
                label[i, j] = k
                if part is not None and piece is not None:
                    part[i, j] = piece
                seeded[i, j] = True
            if not own((i, j)):
                prev = None
                continue
            if prev is not None:
                tw = max(float(width), 1e-6)
                if prev[1] == j and abs(prev[0] - i) == 1:
                    forced_x[min(prev[0], i), j] = max(forced_x[min(prev[0], i), j], tw)
                elif prev[0] == i and abs(prev[1] - j) == 1:
                    forced_y[i, min(prev[1], j)] = max(forced_y[i, min(prev[1], j)], tw)
            elif last is not None and last[:2] != (i, j):
                bridges.append((last[0], last[1], i, j, max(s - last[2], d), float(width)))
            prev, last = (i, j), (i, j, s)
    return bridges


STRIP_SAMPLES = 6    # peec.py:107: lines across each strip's length where its copper's width is measured ...
ADOPT_CELLS = 2      # peec.py:111: ... and how far a cell's copper without a node of its net goes to find one


def _window(lo: float, hi: float, origin: float, d: float, n: int) -> tuple:
    """Grid indices [i0, i1) of the nodes whose cells can hold copper between lo and hi, with two cells of
    margin below and three above (the adoption reach)."""
    return max(int(math.floor((lo - origin) / d)) - 2, 0), min(int(math.ceil((hi - origin) / d)) + 3, n)


def _border_widths(xa, ya, xe, ye, i0: int, wi: int, j0: int, wj: int, x0: float, y0: float, d: float, strips,
                   lead: int):
    """For the strips along x of a window (its cells i0 .. i0+wi, j0 .. j0+wj): the covered length of each
    strip's border line x = x_i + d/2 over d, copper on lines without a strip of the net adopted by the nearest
    strip along the border (within ADOPT_FACES), and the series factor of lone narrow bands from the width at
    STRIP_SAMPLES lines across each strip's length.  The border lines are scanned from the window's lead-th
    border before the strips' first (lead 1: from its left edge, the lines' cover is also every cell's right
    border; lead 0: from the first strip's own line), so the lines fall where the reference puts them.  Returns
    (widths, factors, the cover of every scanned line).  The y strips are the same with x and y swapped."""
    q = STRIP_SAMPLES
    along = ((0, 1), (0, -1))
    lines = line_cover(xa, ya, xe, ye, x0 + (i0 + 0.5 - lead) * d, d, wi - 1 + 2 * lead, y0 + j0 * d, d, wj)
    width = adopt(lines[lead:lead + wi - 1, :] / d, strips, along, ADOPT_FACES)
    cuts = line_cover(xa, ya, xe, ye, x0 + (i0 + 0.5 / q) * d, d / q, (wi - 1) * q, y0 + j0 * d, d, wj) / d
    cuts = cuts.reshape(wi - 1, q, wj)
    samples = [adopt(cuts[:, p, :], strips, along, ADOPT_FACES) for p in range(q)]
    return width, series_factor(width, samples, strips, 1), lines


def exact_copper(nets: list, label: np.ndarray, xb: np.ndarray, yb: np.ndarray, x0: float, y0: float,
                 d: float) -> tuple:
    """Strip widths and node areas measured on the copper itself (GroundTruth's _exact_copper, peec.py:708-771):
    nets[k] = (pa, pb), net k's copper as oriented edges (ring_edges; None: no copper), label the cells' nets,
    xb / yb the strips; returns (ex_x (nx-1, ny), ex_y (nx, ny-1), area (nx, ny), kx, ky): per strip the covered
    length of the cell border it crosses over d (copper of its net on a border line where the net has no strip
    adopted by the nearest strip within ADOPT_FACES), per node its cell's copper of its net over d^2 (adopted
    within ADOPT_CELLS), and per strip of a lone narrow band the series factor of its width measured at
    STRIP_SAMPLES lines along it (1 elsewhere).  Each net is worked in a window of cells around its copper."""
    nx, ny = label.shape
    ex_x, ex_y, area = np.zeros((nx - 1, ny)), np.zeros((nx, ny - 1)), np.zeros((nx, ny))
    kx, ky = np.ones((nx - 1, ny)), np.ones((nx, ny - 1))
    for k, edges in enumerate(nets):
        if edges is None or len(edges[0]) == 0:
            continue
        pa, pb = (np.asarray(e, float).reshape(-1, 2) for e in edges)
        lo, hi = np.minimum(pa.min(0), pb.min(0)), np.maximum(pa.max(0), pb.max(0))
        i0, i1 = _window(lo[0], hi[0], x0, d, nx)
        j0, j1 = _window(lo[1], hi[1], y0, d, ny)
        wi, wj = i1 - i0, j1 - j0
        if wi < 2 or wj < 2:
            continue
        mine = label[i0:i1, j0:j1] == k
        sx = xb[i0:i1 - 1, j0:j1] & mine[:-1, :]
        sy = yb[i0:i1, j0:j1 - 1] & mine[:, :-1]
        wx, fx, borders = _border_widths(pa[:, 0], pa[:, 1], pb[:, 0], pb[:, 1], i0, wi, j0, wj, x0, y0, d, sx, 1)
        wy, fy, _ = _border_widths(pa[:, 1], pa[:, 0], pb[:, 1], pb[:, 0], j0, wj, i0, wi, y0, x0, d, sy.T, 0)
        ex_x[i0:i1 - 1, j0:j1] += wx
        ex_y[i0:i1, j0:j1 - 1] += wy.T
        kx[i0:i1 - 1, j0:j1][sx] = fx[sx]
        ky[i0:i1, j0:j1 - 1][sy] = fy.T[sy]
        cells = cell_areas(pa, pb, x0 + (i0 - 0.5) * d, y0 + (j0 - 0.5) * d, d, wi, wj, borders[1:wi + 1, :]) / (d * d)
        # a cell's copper with no node of its net goes to the nearest node that has one, across rows first
        area[i0:i1, j0:j1] += adopt(np.clip(cells, 0.0, 1.0), mine, ((1, 0), (-1, 0), (0, 1), (0, -1)), ADOPT_CELLS)
    return ex_x, ex_y, area, kx, ky


def coarse_from_fine(nets: list, x0: float, y0: float, d: float, nx: int, ny: int, s: int) -> tuple:
    """Cells, their nets and the copper joining neighbours from a sub-grid of pitch d / s (GroundTruth's
    _coarse_from_fine, peec.py:774-849).  nets[k] = net k's copper (a polygon (outline, holes), a list of them, or
    None), points of the sub-grid inside it (strictly, holes closed: synth.copper_at) take the first net that holds them.
    Returns (label (nx, ny): each cell's net, its largest piece of one net's sub-grid copper inside the cell when
    that spans at least s sub-grid points, else -1; cross_x (nx-1, ny) / cross_y (nx, ny-1): the fraction of
    the s sub-grid strips across the border two cells' kept pieces join by; fill (nx, ny): the kept piece's share
    of the cell; off_x / off_y: the crossing strips' mean position along the border from its middle, over d)."""
    from .synth import copper_at
    df = d / s
    mx, my = nx * s, ny * s
    xf = x0 - 0.5 * d + (np.arange(mx) + 0.5) * df
    yf = y0 - 0.5 * d + (np.arange(my) + 0.5) * df
    fine = np.full((mx, my), -1, np.int64)
    for k, poly in enumerate(nets):
        if poly is None:
            continue
        polys = polygons_of(poly)
        pts = np.concatenate([np.asarray(o, float) for o, _ in polys])
        a = np.searchsorted(xf, pts[:, 0].min(), "left"), np.searchsorted(xf, pts[:, 0].max(), "right")
        b = np.searchsorted(yf, pts[:, 1].min(), "left"), np.searchsorted(yf, pts[:, 1].max(), "right")
        if a[0] >= a[1] or b[0] >= b[1]:
            continue
        X, Y = np.meshgrid(xf[a[0]:a[1]], yf[b[0]:b[1]], indexing="ij")
        hit = np.zeros(X.shape, bool)
        for outline, holes in polys:
            hit |= copper_at(X, Y, np.asarray(outline, float), [np.asarray(q, float) for q in holes])
        win = fine[a[0]:a[1], b[0]:b[1]]
        win[hit & (win < 0)] = k
    cu = fine >= 0
    # pieces: sub-grid points of one net joined inside their cell (4-neighbours), named by their least flat
    # index through min-label propagation (the join never crosses a cell border)
    lab = np.where(cu, np.arange(mx * my).reshape(mx, my), np.iinfo(np.int64).max)
    join_x = cu[:-1, :] & (fine[:-1, :] == fine[1:, :]) & ((np.arange(1, mx) % s) != 0)[:, None]
    join_y = cu[:, :-1] & (fine[:, :-1] == fine[:, 1:]) & ((np.arange(1, my) % s) != 0)[None, :]
    while True:
        new = lab.copy()
        np.minimum(new[:-1, :], np.where(join_x, lab[1:, :], new[:-1, :]), out=new[:-1, :])
        np.minimum(new[1:, :], np.where(join_x, lab[:-1, :], new[1:, :]), out=new[1:, :])
        np.minimum(new[:, :-1], np.where(join_y, lab[:, 1:], new[:, :-1]), out=new[:, :-1])
        np.minimum(new[:, 1:], np.where(join_y, lab[:, :-1], new[:, 1:]), out=new[:, 1:])
        if np.array_equal(new, lab):
            break
        lab = new
    size = np.bincount(lab[cu], minlength=mx * my)
    cell = (np.arange(mx) // s)[:, None] * ny + (np.arange(my) // s)[None, :]
    # each cell keeps its largest piece (the least name of equals) when it spans at least s points
    names = np.flatnonzero(size)
    cell_of = cell.ravel()[names]
    order = np.lexsort((names, -size[names], cell_of))
    first = np.r_[True, cell_of[order][1:] != cell_of[order][:-1]]
    best = names[order][first]
    best = best[size[best] >= s]
    label = np.full(nx * ny, -1, np.int64)
    label[cell.ravel()[best]] = fine.ravel()[best]
    fill = np.zeros(nx * ny)
    fill[cell.ravel()[best]] = size[best] / (s * s)
    kept = np.zeros(mx * my, bool)
    kept[best] = True
    on = cu & kept[np.where(cu, lab, 0)]

    def crossings(hit, coarse, along, shape):
        """Sub-grid strips joining two kept pieces across cell borders: per coarse strip their count over s
        and their mean position along the border from its middle, over d."""
        i, j = np.nonzero(hit)
        ci, cj = coarse(i, j)
        pos = along(i, j) % s
        count = np.zeros(shape)
        spread = np.zeros(shape)
        np.add.at(count, (ci, cj), 1.0)
        np.add.at(spread, (ci, cj), 2.0 * pos + 1.0 - s)
        with np.errstate(invalid="ignore", divide="ignore"):
            off = np.where(count > 0, spread / (2.0 * s * count), 0.0)
        return count / s, off
    rows_x = np.arange(s - 1, mx - 1, s)                  # sub-rows whose next sub-row is in the next cell
    cols_y = np.arange(s - 1, my - 1, s)
    hit_x = on[rows_x, :] & on[rows_x + 1, :] & (fine[rows_x, :] == fine[rows_x + 1, :])
    hit_y = on[:, cols_y] & on[:, cols_y + 1] & (fine[:, cols_y] == fine[:, cols_y + 1])
    cx, ox = crossings(hit_x, lambda i, j: (i, j // s), lambda i, j: j, (nx - 1, ny))
    cy, oy = crossings(hit_y, lambda i, j: (i // s, j), lambda i, j: i, (nx, ny - 1))
    return label.reshape(nx, ny), cx, cy, fill.reshape(nx, ny), ox, oy



PIECE_TOL = 0.005    # peec.py:106: copper of one net within this of itself (mm) is one piece (touching fills)


def polygons_of(piece) -> list:
    """A piece's polygons: a polygon (outline, holes) alone (its outline's first vertex a pair of numbers), or a
    list of them."""
    return [piece] if np.isscalar(piece[0][0][0]) else list(piece)


def _segment_distance(a0, a1, b0, b1) -> np.ndarray:
    """Distances between 2D segments a0-a1 (n, 2) and b0-b1 (m, 2), all pairs (n, m): 0 where they cross, else
    the least of the four end-to-segment distances."""
    def to_segment(p, q0, q1):
        d = q1 - q0
        t = np.clip(np.einsum("nmk,mk->nm", p[:, None, :] - q0[None], d) / np.maximum(np.einsum("mk,mk->m", d, d),
                                                                                      1e-300), 0.0, 1.0)
        return np.hypot(*np.moveaxis(p[:, None, :] - (q0[None] + t[..., None] * d[None]), -1, 0))

    def cross(o, p, q):
        return (p[..., 0] - o[..., 0]) * (q[..., 1] - o[..., 1]) - (p[..., 1] - o[..., 1]) * (q[..., 0] - o[..., 0])
    A0, A1, B0, B1 = a0[:, None], a1[:, None], b0[None], b1[None]
    hit = ((cross(A0, A1, B0) * cross(A0, A1, B1) < 0) & (cross(B0, B1, A0) * cross(B0, B1, A1) < 0))
    dist = np.minimum(np.minimum(to_segment(a0, b0, b1), to_segment(a1, b0, b1)),
                      np.minimum(to_segment(b0, a0, a1).T, to_segment(b1, a0, a1).T))
    return np.where(hit, 0.0, dist)


def _polygon_distance(p, q) -> float:
    """The distance between two polygons (outline, holes): 0 where their copper meets or one holds the other's
    outline, else the least distance between their rings."""
    pa, pb = ring_edges(*p)
    qa, qb = ring_edges(*q)
    if bool(_covers(qa[:1, 0], qa[:1, 1], p)[0]) or bool(_covers(pa[:1, 0], pa[:1, 1], q)[0]):
        return 0.0
    return float(_segment_distance(pa, pb, qa, qb).min())


def pieces(polygons: list, tol: float = PIECE_TOL) -> list:
    """One net's polygons grouped into its connected pieces of copper (GroundTruth's _pieces, peec.py:852-873):
    polygons that meet or lie within tol of each other (transitively) are one piece, a list of polygons; a lone
    polygon is a piece by itself.  The polygons are those of the net's union (not overlapping)."""
    n = len(polygons)
    if n <= 1:
        return [p for p in polygons]
    group = list(range(n))

    def root(i):
        while group[i] != i:
            group[i] = group[group[i]]
            i = group[i]
        return i
    box = [(np.min(np.asarray(o, float), axis=0) - tol, np.max(np.asarray(o, float), axis=0) + tol) for o, _ in polygons]
    for i in range(n):
        for j in range(i + 1, n):
            if np.any(box[i][1] < box[j][0]) or np.any(box[j][1] < box[i][0]):
                continue
            if root(i) != root(j) and _polygon_distance(polygons[i], polygons[j]) <= tol:
                group[max(root(i), root(j))] = min(root(i), root(j))
    out = {}
    for i in range(n):
        out.setdefault(root(i), []).append(polygons[i])
    return [members[0] if len(members) == 1 else members for members in out.values()]


def _covers(px, py, piece) -> np.ndarray:
    """Points inside a piece's copper or on its border (shapely's covers)."""
    from .synth import polygon_contains
    out = np.zeros(np.shape(px), bool)
    for outline, holes in polygons_of(piece):
        ins, on = polygon_contains(px, py, np.asarray(outline, float))
        cov = ins | on
        for h in holes:
            hin, _ = polygon_contains(px, py, np.asarray(h, float))
            cov &= ~hin
        out |= cov
    return out


def _inside(X, Y, pieces: list) -> np.ndarray:
    """Points strictly inside any of the pieces (outline minus closed holes)."""
    from .synth import copper_at
    out = np.zeros(np.shape(X), bool)
    for piece in pieces:
        for outline, holes in polygons_of(piece):
            out |= copper_at(X, Y, np.asarray(outline, float), [np.asarray(h, float) for h in holes])
    return out


@dataclass
class LayerRaster:
    """One layer's copper on a grid of pitch d (GroundTruth's Grid, peec.py:197-223, without the heat points):
    nodes, strips, each node's net (label, -1: none), the cells' copper fraction (sub-grid only), the tracks'
    bridges, and with a sub-grid the strips' widths, offsets and resistance widths and the nodes' areas."""
    x0: float
    y0: float
    d: float
    nx: int
    ny: int
    node: np.ndarray
    xb: np.ndarray
    yb: np.ndarray
    label: np.ndarray
    nets: list
    fill: Optional[np.ndarray] = None
    bridges: list = field(default_factory=list)
    wx: Optional[np.ndarray] = None
    wy: Optional[np.ndarray] = None
    ox: Optional[np.ndarray] = None
    oy: Optional[np.ndarray] = None
    area: Optional[np.ndarray] = None
    rx: Optional[np.ndarray] = None
    ry: Optional[np.ndarray] = None

    def widths(self) -> Optional[dict]:
        """The strip widths as the solver's Grid takes them (None: every strip full)."""
        if self.wx is None:
            return None
        return {"wx": self.wx, "wy": self.wy, "ox": self.ox, "oy": self.oy, "rx": self.rx, "ry": self.ry}


def build_layer(nets: dict, bbox: tuple, d: float, seeds: Optional[dict] = None, lines: Optional[dict] = None,
                sub: int = 1) -> LayerRaster:
    """A layer's copper on a grid of pitch d over bbox (x0, y0, x1, y1) (GroundTruth's build_grid,
    peec.py:329-449, heat points left out).  nets {net: [piece, ...]}: each net's copper as its connected pieces
    (a polygon (outline, holes) or a list of polygons, in the unit of d; pieces() groups a net's polygons); seeds {net: [(x, y)]}: points whose nearest free node becomes
    the net's (a via ring or pad smaller than the grid); lines {net: [(polyline, width)]}: tracks claimed by
    rasterise_tracks.  sub = 1: a node is a net's when its point lies inside the net's copper (the first net
    keeps it), a strip when its midpoint does too; sub > 1: cells, joins and offsets from the sub-grid
    (coarse_from_fine, pieces kept apart), then the widths and areas from the copper itself (exact_copper,
    strip_widths; the resistance width times the series factor).  A strip joins two nodes of one net and one
    piece whose midpoint is that net's copper, or either of which is seeded, or that a track forces."""
    x0, y0, x1, y1 = bbox
    nx = max(int(math.ceil((x1 - x0) / d)) + 1, 3)
    ny = max(int(math.ceil((y1 - y0) / d)) + 1, 3)
    names = list(nets)
    per_net = [list(nets[n]) for n in names]
    fine = sub > 1
    pieces = [(k, p) for k, ps in enumerate(per_net) for p in ps] if fine else []
    fill = None
    if fine:
        part, cross_x, cross_y, fill, off_x, off_y = coarse_from_fine([p for _, p in pieces], x0, y0, d, nx, ny, sub)
        label = np.array([k for k, _ in pieces] + [-1], int)[part]
        mids_x = np.where(cross_x > 0, label[:-1, :], -1)
        mids_y = np.where(cross_y > 0, label[:, :-1], -1)
    else:
        label = -np.ones((nx, ny), int)
        mids_x, mids_y = np.full((nx - 1, ny), -1), np.full((nx, ny - 1), -1)
        part = None
        xs, ys = x0 + np.arange(nx) * d, y0 + np.arange(ny) * d
        for k, ps in enumerate(per_net):
            if not ps:
                continue
            outlines = [np.asarray(o, float) for piece in ps for o, _ in polygons_of(piece)]
            lo = np.min([o.min(axis=0) for o in outlines], axis=0)
            hi = np.max([o.max(axis=0) for o in outlines], axis=0)
            i0, i1 = max(int(math.floor((lo[0] - x0) / d)) - 1, 0), min(int(math.ceil((hi[0] - x0) / d)) + 2, nx)
            j0, j1 = max(int(math.floor((lo[1] - y0) / d)) - 1, 0), min(int(math.ceil((hi[1] - y0) / d)) + 2, ny)
            if i0 >= i1 or j0 >= j1:
                continue
            X, Y = np.meshgrid(xs[i0:i1], ys[j0:j1], indexing="ij")
            win = label[i0:i1, j0:j1]
            win[_inside(X, Y, ps) & (win < 0)] = k
            mx = mids_x[i0:min(i1, nx - 1), j0:j1]
            mx[_inside(X[: mx.shape[0]] + d / 2, Y[: mx.shape[0]], ps) & (mx < 0)] = k
            my = mids_y[i0:i1, j0:min(j1, ny - 1)]
            my[_inside(X[:, : my.shape[1]], Y[:, : my.shape[1]] + d / 2, ps) & (my < 0)] = k
    if part is None:
        part = label                      # no pieces: a net is its own piece (the same array)

    def piece_at(k: int, px: float, py: float) -> int:
        """The piece of net k holding (px, py) (inside or on its border), else a new piece of its own."""
        if not pieces:
            return k
        for c, (net, poly) in enumerate(pieces):
            if net == k and poly is not None and bool(_covers(np.array([px]), np.array([py]), poly)[0]):
                return c
        pieces.append((k, None))
        return len(pieces) - 1

    seeded = np.zeros((nx, ny), bool)
    for net, points in (seeds or {}).items():
        if net not in names:
            continue
        k = names.index(net)
        for px, py in points:
            i, j = int(round((px - x0) / d)), int(round((py - y0) / d))
            if 0 <= i < nx and 0 <= j < ny and label[i, j] < 0:
                label[i, j] = k
                part[i, j] = piece_at(k, px, py)
                seeded[i, j] = True
    forced_x, forced_y = np.zeros((nx - 1, ny)), np.zeros((nx, ny - 1))
    bridges = []
    for net, polylines in (lines or {}).items():
        if net not in names:
            continue
        k = names.index(net)
        owners = None
        if pieces:
            owners = []
            for pts, _ in polylines:
                (ax, ay), (bx, by) = pts[0], pts[1] if len(pts) > 1 else pts[0]
                owners.append(piece_at(k, (ax + bx) / 2, (ay + by) / 2))
        bridges += rasterise_tracks(k, polylines, x0, y0, d, label, seeded, forced_x, forced_y, part, owners)
    xb = (label[:-1, :] >= 0) & (label[:-1, :] == label[1:, :]) & (part[:-1, :] == part[1:, :]) & (
        (mids_x == label[:-1, :]) | seeded[:-1, :] | seeded[1:, :] | (forced_x > 0))
    yb = (label[:, :-1] >= 0) & (label[:, :-1] == label[:, 1:]) & (part[:, :-1] == part[:, 1:]) & (
        (mids_y == label[:, :-1]) | seeded[:, :-1] | seeded[:, 1:] | (forced_y > 0))
    out = LayerRaster(x0, y0, d, nx, ny, label >= 0, xb, yb, label, names, fill, bridges)
    if fine:
        edges = []
        for ps in per_net:
            rings = [ring_edges(o, h) for piece in ps for o, h in polygons_of(piece)]
            edges.append((np.concatenate([a for a, _ in rings]), np.concatenate([b for _, b in rings]))
                         if rings else None)
        ex_x, ex_y, area, kx, ky = exact_copper(edges, label, xb, yb, x0, y0, d)
        out.wx, out.ox = strip_widths(xb, cross_x, off_x, forced_x, d, ex_x)
        out.wy, out.oy = strip_widths(yb, cross_y, off_y, forced_y, d, ex_y)
        out.area, out.rx, out.ry = area, out.wx * kx, out.wy * ky
    return out
