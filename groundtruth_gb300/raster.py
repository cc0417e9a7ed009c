"""The exact-copper raster's arithmetic (GroundTruth: peec.py:482-705, the parts of build_grid's exact-copper pass
that need no polygon library): how much copper crosses each cell border along scanlines, the copper area of each
cell from its outline by Green's theorem, a strip's width and centre from those, copper of a border without a strip
of its net moved to the nearest strip that has one, and the series factor of a narrow run whose width changes
along its length; and the walk that claims tracks' cells and strips on a layer's grid (peec.py:893-983).  Polygons are given as their edges (outlines counter-clockwise, holes clockwise: ring_edges), in
the same length unit as the pitch."""
from __future__ import annotations

import math
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
