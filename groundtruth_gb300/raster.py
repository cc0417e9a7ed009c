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


def line_cover(ua, va, ub, vb, u0: float, du: float, n_lines: int, v0: float, d: float, n_cells: int) -> np.ndarray:
    """(n_lines, n_cells): on each line u = u0 + m du the length of each interval [v0 + (c - 1/2) d, v0 + (c + 1/2) d]
    inside the polygons with edges (ua, va) -> (ub, vb) (peec.py:533-580).  A scanline: an edge crosses the lines
    with u in [min, max) of its ends (half open: a vertex on a line counts once, an edge along one not at all),
    each line's crossings sorted along it bound the inside in pairs, each inside span adds its overlap with every
    interval; a line with an odd number of crossings is skipped."""
    out = np.zeros((n_lines, n_cells))
    ua, va, ub, vb = (np.asarray(x, float) for x in (ua, va, ub, vb))
    if len(ua) == 0 or n_lines <= 0 or n_cells <= 0:
        return out
    lo, hi = np.minimum(ua, ub), np.maximum(ua, ub)
    first = np.clip(np.ceil((lo - u0) / du), 0, n_lines).astype(np.int64)
    last = np.clip(np.ceil((hi - u0) / du), 0, n_lines).astype(np.int64)
    edges = np.flatnonzero(last > first)
    if len(edges) == 0:
        return out
    cnt = (last - first)[edges]
    e = np.repeat(edges, cnt)
    line = np.repeat(first[edges], cnt) + (np.arange(int(cnt.sum())) - np.repeat(np.cumsum(cnt) - cnt, cnt))
    u = u0 + line * du
    v = va[e] + (u - ua[e]) * (vb[e] - va[e]) / (ub[e] - ua[e])
    order = np.lexsort((v, line))
    line, v = line[order], v[order]
    per_line = np.bincount(line, minlength=n_lines)
    pos = np.arange(len(line)) - np.searchsorted(line, line)
    opens = np.flatnonzero((pos % 2 == 0) & (per_line[line] % 2 == 0))
    ln, a, b = line[opens], v[opens], v[opens + 1]
    base, span = v0 - d / 2, n_cells * d
    a, b = np.clip(a - base, 0.0, span), np.clip(b - base, 0.0, span)
    keep = b > a
    ln, a, b = ln[keep], a[keep], b[keep]
    ca = np.minimum((a / d).astype(np.int64), n_cells - 1)
    cb = np.minimum((b / d).astype(np.int64), n_cells - 1)
    size = n_lines * n_cells
    flat = out.reshape(-1)
    inside = ca == cb
    flat += np.bincount(ln[inside] * n_cells + ca[inside], b[inside] - a[inside], size)
    cross = ~inside
    l2, a2, b2, ca2, cb2 = ln[cross], a[cross], b[cross], ca[cross], cb[cross]
    flat += np.bincount(l2 * n_cells + ca2, (ca2 + 1) * d - a2, size)
    flat += np.bincount(l2 * n_cells + cb2, b2 - cb2 * d, size)
    # whole intervals between a span's first and last: +d from ca + 1, -d from cb, summed along the line
    steps = np.zeros((n_lines, n_cells + 1))
    w = n_lines * (n_cells + 1)
    steps.reshape(-1)[:] += np.bincount(l2 * (n_cells + 1) + ca2 + 1, np.full(len(l2), d), w)
    steps.reshape(-1)[:] -= np.bincount(l2 * (n_cells + 1) + cb2, np.full(len(l2), d), w)
    out += np.cumsum(steps, axis=1)[:, :n_cells]
    return out


def cell_areas(pa, pb, xl: float, yl: float, d: float, wi: int, wj: int, right: np.ndarray) -> np.ndarray:
    """(wi, wj): the copper area of each cell [xl + i d, xl + (i+1) d] x [yl + j d, yl + (j+1) d] inside the
    polygons with oriented edges pa -> pb, `right` the covered length of each cell's right border
    (peec.py:583-622).  Green's theorem, area = closed integral of x dy: the edges cut at every grid line, each
    piece adds (its mean x - the cell's left) dy to its cell; the cell's own right border adds d times its
    covered length."""
    out = np.zeros((wi, wj))
    pa, pb = np.asarray(pa, float).reshape(-1, 2), np.asarray(pb, float).reshape(-1, 2)
    if len(pa):
        xa, ya, xb, yb = pa[:, 0], pa[:, 1], pb[:, 0], pb[:, 1]
        ts, es = [np.zeros(len(xa)), np.ones(len(xa))], [np.arange(len(xa))] * 2
        for a, b, origin, n in ((xa, xb, xl, wi + 1), (ya, yb, yl, wj + 1)):
            lo, hi = np.minimum(a, b), np.maximum(a, b)
            m0 = np.clip(np.ceil((lo - origin) / d), 0, n).astype(np.int64)
            m1 = np.clip(np.ceil((hi - origin) / d), 0, n).astype(np.int64)
            sel = np.flatnonzero(m1 > m0)
            cnt = (m1 - m0)[sel]
            e = np.repeat(sel, cnt)
            m = np.repeat(m0[sel], cnt) + (np.arange(int(cnt.sum())) - np.repeat(np.cumsum(cnt) - cnt, cnt))
            ts.append((origin + m * d - a[e]) / (b[e] - a[e]))
            es.append(e)
        t, e = np.concatenate(ts), np.concatenate(es)
        order = np.lexsort((t, e))
        t, e = t[order], e[order]
        piece = e[1:] == e[:-1]
        e, t0, t1 = e[:-1][piece], t[:-1][piece], t[1:][piece]
        x0, y0 = xa[e] + t0 * (xb[e] - xa[e]), ya[e] + t0 * (yb[e] - ya[e])
        x1, y1 = xa[e] + t1 * (xb[e] - xa[e]), ya[e] + t1 * (yb[e] - ya[e])
        i = np.floor(((x0 + x1) / 2 - xl) / d).astype(np.int64)
        j = np.floor(((y0 + y1) / 2 - yl) / d).astype(np.int64)
        ok = (i >= 0) & (i < wi) & (j >= 0) & (j < wj)
        add = ((x0 + x1) / 2 - (xl + i * d)) * (y1 - y0)
        out.reshape(-1)[:] += np.bincount(i[ok] * wj + j[ok], add[ok], wi * wj)
    return out + d * np.asarray(right, float)


def strip_widths(exists, cross, offset, forced, d: float, exact=None) -> tuple:
    """Each strip's copper width as a fraction of the pitch and its centre's offset across the strip
    (peec.py:482-513): the exact covered border where measured (at most 3 pitches: a strip carries the sliver
    beside it too), else the share of its border the sub-grid saw copper cross, at least a forced track's own
    width, 1 where neither; the centre kept inside the cell; 0 where no strip exists."""
    exists = np.asarray(exists, bool)
    w = np.where(forced > 0, np.maximum(cross, np.minimum(forced / d, 1.0)), cross)
    w = np.where(w > 0, np.minimum(w, 1.0), 1.0)
    if exact is not None:
        w = np.where(exact > 0, np.minimum(exact, 3.0), w)
    o = np.where(cross > 0, offset, 0.0)
    lim = np.maximum((1.0 - w) / 2, 0.0)
    return np.where(exists, w, 0.0), np.where(exists, np.clip(o, -lim, lim), 0.0)


def adopt(cov, has, steps, reach: int = 1) -> np.ndarray:
    """`cov` where `has`, plus the values where nothing of the net exists moved to the nearest place that has one
    along the offsets `steps` within `reach` steps (of two at one distance, the one with more copper of its own);
    values with none within reach are dropped (peec.py:625-656)."""
    cov, has = np.asarray(cov, float), np.asarray(has, bool)
    own = np.where(has, cov, 0.0)
    stray = np.where(has, 0.0, cov)
    out = own.copy()
    ni, nj = cov.shape

    def shifted(di, dj):
        src = (slice(max(di, 0), ni + min(di, 0)), slice(max(dj, 0), nj + min(dj, 0)))
        dst = (slice(max(-di, 0), ni + min(-di, 0)), slice(max(-dj, 0), nj + min(-dj, 0)))
        return src, dst
    for k in range(1, reach + 1):
        if not np.any(stray > 0):
            break
        best = np.full(cov.shape, -1.0)
        pick = np.full(cov.shape, -1)
        for q, (di, dj) in enumerate(steps):
            src, dst = shifted(di * k, dj * k)
            nb_has, nb_cov = np.zeros(cov.shape, bool), np.zeros(cov.shape)
            nb_has[dst], nb_cov[dst] = has[src], own[src]
            better = (stray > 0) & nb_has & (nb_cov > best)
            best = np.where(better, nb_cov, best)
            pick = np.where(better, q, pick)
        for q, (di, dj) in enumerate(steps):
            dst, src = shifted(di * k, dj * k)
            moved = np.where(pick == q, stray, 0.0)
            out[dst] += moved[src]
        stray = np.where(pick >= 0, 0.0, stray)
    return out


def series_factor(face, samples: list, has, axis: int) -> np.ndarray:
    """Per strip, the conductance change of its band (a run of side-by-side strips in one column, `axis` 1: x
    strips by rows, 0: y strips by columns) when the copper's width is taken along the strips' length instead of at
    the border: the harmonic mean of the band's total width at the sample lines over its total at the border, for a
    lone narrow band only (at most BAND_STRIPS strips, no other strip of the net within 2 ADOPT_FACES along the
    border, copper at every sample line); 1 otherwise (peec.py:659-705)."""
    has = np.asarray(has, bool)
    h = has if axis == 1 else has.T
    if not h.any():
        return np.ones(has.shape)
    f_ = np.asarray(face, float) if axis == 1 else np.asarray(face, float).T
    rows = [np.asarray(s, float) if axis == 1 else np.asarray(s, float).T for s in samples]
    n0, n1 = h.shape
    start = h & ~np.concatenate([np.zeros((n0, 1), bool), h[:, :-1]], axis=1)
    run = np.cumsum(start, axis=1) - 1
    r_i, c_i = np.nonzero(h)
    key = r_i * n1 + run[r_i, c_i]
    nk = n0 * n1
    total = np.bincount(key, f_[h], nk)
    size = np.bincount(key, minlength=nk)
    far = n1 + 2 * ADOPT_FACES + 2
    step = np.where(np.r_[True, r_i[1:] != r_i[:-1]], far, np.r_[far, c_i[1:] - c_i[:-1]])
    head = step != 1
    gap_before = np.full(nk, far)
    gap_before[key[head]] = step[head] - 1
    gap_after = np.where(np.r_[size[1:] > 0, False], np.r_[gap_before[1:], far], far)
    lone = (size <= BAND_STRIPS) & (gap_before > 2 * ADOPT_FACES) & (gap_after > 2 * ADOPT_FACES)
    inv, seen = np.zeros(nk), np.ones(nk, bool)
    for srow in rows:
        t = np.bincount(key, srow[h], nk)
        seen &= t > 0
        inv += 1.0 / np.maximum(t, 1e-300)
    harmonic = len(rows) / np.maximum(inv, 1e-300)
    factor = np.where(lone & seen & (total > 0), harmonic / np.maximum(total, 1e-300), 1.0)
    out = np.ones(h.shape)
    out[h] = factor[key]
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


def _bounds(pa: np.ndarray, pb: np.ndarray) -> tuple:
    lo = np.minimum(pa.min(axis=0), pb.min(axis=0))
    hi = np.maximum(pa.max(axis=0), pb.max(axis=0))
    return float(lo[0]), float(lo[1]), float(hi[0]), float(hi[1])


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
    along_rows, along_cols = ((0, 1), (0, -1)), ((1, 0), (-1, 0))
    q = STRIP_SAMPLES
    for k, edges in enumerate(nets):
        if edges is None or len(edges[0]) == 0:
            continue
        pa, pb = edges
        bx0, by0, bx1, by1 = _bounds(pa, pb)
        i0, i1 = max(int(math.floor((bx0 - x0) / d)) - 2, 0), min(int(math.ceil((bx1 - x0) / d)) + 3, nx)
        j0, j1 = max(int(math.floor((by0 - y0) / d)) - 2, 0), min(int(math.ceil((by1 - y0) / d)) + 3, ny)
        wi, wj = i1 - i0, j1 - j0
        if wi < 2 or wj < 2:
            continue
        xa, ya, xe, ye = pa[:, 0], pa[:, 1], pb[:, 0], pb[:, 1]
        # vertical borders x = x_i - d/2 (line m: the left border of window column m) and horizontal ones
        # y = y_j + d/2 between window rows: the copper each cell's stretch of them holds
        vert = line_cover(xa, ya, xe, ye, x0 + (i0 - 0.5) * d, d, wi + 1, y0 + j0 * d, d, wj)
        horiz = line_cover(ya, xa, ye, xe, y0 + (j0 + 0.5) * d, d, wj - 1, x0 + i0 * d, d, wi).T
        mine = label[i0:i1, j0:j1] == k
        sx = xb[i0:i1 - 1, j0:j1] & mine[:-1, :]
        sy = yb[i0:i1, j0:j1 - 1] & mine[:, :-1]
        fx = adopt(vert[1:wi, :] / d, sx, along_rows, ADOPT_FACES)
        fy = adopt(horiz / d, sy, along_cols, ADOPT_FACES)
        ex_x[i0:i1 - 1, j0:j1] += fx
        ex_y[i0:i1, j0:j1 - 1] += fy
        # the width along each strip: q lines across its length at x_i + (p + 1/2) d / q
        cut_x = (line_cover(xa, ya, xe, ye, x0 + (i0 + 0.5 / q) * d, d / q, (wi - 1) * q, y0 + j0 * d, d, wj)
                 / d).reshape(wi - 1, q, wj)
        cut_y = (line_cover(ya, xa, ye, xe, y0 + (j0 + 0.5 / q) * d, d / q, (wj - 1) * q, x0 + i0 * d, d, wi)
                 / d).reshape(wj - 1, q, wi)
        samples_x = [adopt(cut_x[:, p, :], sx, along_rows, ADOPT_FACES) for p in range(q)]
        samples_y = [adopt(cut_y[:, p, :].T, sy, along_cols, ADOPT_FACES) for p in range(q)]
        kx[i0:i1 - 1, j0:j1][sx] = series_factor(fx, samples_x, sx, 1)[sx]
        ky[i0:i1, j0:j1 - 1][sy] = series_factor(fy, samples_y, sy, 0)[sy]
        cells = cell_areas(pa, pb, x0 + (i0 - 0.5) * d, y0 + (j0 - 0.5) * d, d, wi, wj, vert[1:wi + 1, :]) / (d * d)
        area[i0:i1, j0:j1] += adopt(np.clip(cells, 0.0, 1.0), mine, along_cols + along_rows, ADOPT_CELLS)
    return ex_x, ex_y, area, kx, ky


def coarse_from_fine(nets: list, x0: float, y0: float, d: float, nx: int, ny: int, s: int) -> tuple:
    """Cells, their nets and the copper joining neighbours from a sub-grid of pitch d / s (GroundTruth's
    _coarse_from_fine, peec.py:774-849).  nets[k] = net k's copper (a polygon (outline, holes), a list of them, or
    None), points of the sub-grid inside it (strictly, holes closed: synth.copper_at) take the first net that holds them.
    Returns (label (nx, ny): each cell's net, its largest piece of one net's sub-grid copper inside the cell when
    that spans at least s sub-grid points, else -1; cross_x (nx-1, ny) / cross_y (nx, ny-1): the fraction of
    the s sub-grid strips across the border two cells' kept pieces join by; fill (nx, ny): the kept piece's share
    of the cell; off_x / off_y: the crossing strips' mean position along the border from its middle, over d)."""
    from scipy.sparse.csgraph import connected_components
    import scipy.sparse as sp
    from .synth import copper_at
    df = d / s
    mx, my = nx * s, ny * s
    xf = x0 - d / 2 + (np.arange(mx) + 0.5) * df
    yf = y0 - d / 2 + (np.arange(my) + 0.5) * df
    fine = -np.ones((mx, my), np.int32)
    for k, poly in enumerate(nets):
        if poly is None:
            continue
        polys = polygons_of(poly)
        bx0, by0 = np.min([np.min(np.asarray(o, float), axis=0) for o, _ in polys], axis=0)
        bx1, by1 = np.max([np.max(np.asarray(o, float), axis=0) for o, _ in polys], axis=0)
        p0, p1 = max(int(math.floor((bx0 - xf[0]) / df)) - 1, 0), min(int(math.ceil((bx1 - xf[0]) / df)) + 2, mx)
        q0, q1 = max(int(math.floor((by0 - yf[0]) / df)) - 1, 0), min(int(math.ceil((by1 - yf[0]) / df)) + 2, my)
        if p0 >= p1 or q0 >= q1:
            continue
        X, Y = np.meshgrid(xf[p0:p1], yf[q0:q1], indexing="ij")
        win = fine[p0:p1, q0:q1]
        inside = np.zeros(X.shape, bool)
        for outline, holes in polys:
            inside |= copper_at(X, Y, np.asarray(outline, float), [np.asarray(h, float) for h in holes])
        win[inside & (win < 0)] = k
    same_x = (fine[:-1, :] >= 0) & (fine[:-1, :] == fine[1:, :])         # sub-grid strips within one net
    same_y = (fine[:, :-1] >= 0) & (fine[:, :-1] == fine[:, 1:])
    border_x = ((np.arange(mx - 1) + 1) % s == 0)[:, None]                # ... that cross a cell border
    border_y = ((np.arange(my - 1) + 1) % s == 0)[None, :]
    n = mx * my
    at = np.arange(n).reshape(mx, my)
    inner_x, inner_y = same_x & ~border_x, same_y & ~border_y           # the cells' pieces: strips inside cells
    a = np.concatenate([at[:-1, :][inner_x], at[:, :-1][inner_y]])
    b = np.concatenate([at[1:, :][inner_x], at[:, 1:][inner_y]])
    _, piece = connected_components(sp.coo_matrix((np.ones(len(a), np.int8), (a, b)), shape=(n, n)), directed=False)
    piece = piece.reshape(mx, my)
    cell_of = (np.arange(mx) // s)[:, None] * ny + (np.arange(my) // s)[None, :]
    cu = fine >= 0
    pid = piece[cu]
    size = np.bincount(pid, minlength=n)
    p_cell, p_net = np.full(n, -1), np.full(n, -1)
    p_cell[pid] = cell_of[cu]
    p_net[pid] = fine[cu]
    pieces = np.unique(pid)
    pieces = pieces[np.lexsort((-size[pieces], p_cell[pieces]))]           # per cell, the largest piece first
    lead = np.ones(len(pieces), bool)
    lead[1:] = p_cell[pieces[1:]] != p_cell[pieces[:-1]]
    kept = pieces[lead]
    kept = kept[size[kept] >= s]
    label = -np.ones(nx * ny, int)
    label[p_cell[kept]] = p_net[kept]
    fill = np.zeros(nx * ny)
    fill[p_cell[kept]] = size[kept] / (s * s)
    is_kept = np.zeros(n, bool)
    is_kept[kept] = True
    on = cu & is_kept[piece]
    cross_x, off_x = np.zeros((nx - 1, ny)), np.zeros((nx - 1, ny))
    fi, fj = np.nonzero(same_x & border_x & on[:-1, :] & on[1:, :])
    np.add.at(cross_x, (fi // s, fj // s), 1.0 / s)
    np.add.at(off_x, (fi // s, fj // s), ((fj % s + 0.5) / s - 0.5) / s)
    cross_y, off_y = np.zeros((nx, ny - 1)), np.zeros((nx, ny - 1))
    fi, fj = np.nonzero(same_y & border_y & on[:, :-1] & on[:, 1:])
    np.add.at(cross_y, (fi // s, fj // s), 1.0 / s)
    np.add.at(off_y, (fi // s, fj // s), ((fi % s + 0.5) / s - 0.5) / s)
    with np.errstate(invalid="ignore", divide="ignore"):
        off_x = np.where(cross_x > 0, off_x / cross_x, 0.0)
        off_y = np.where(cross_y > 0, off_y / cross_y, 0.0)
    return label.reshape(nx, ny), cross_x, cross_y, fill.reshape(nx, ny), off_x, off_y


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
