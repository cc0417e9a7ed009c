"""The exact-copper raster's arithmetic (GroundTruth: peec.py:482-705, the parts of build_grid's exact-copper pass
that need no polygon library): how much copper crosses each cell border along scanlines, the copper area of each
cell from its outline by Green's theorem, a strip's width and centre from those, copper of a border without a strip
of its net moved to the nearest strip that has one, and the series factor of a narrow run whose width changes
along its length.  Polygons are given as their edges (outlines counter-clockwise, holes clockwise: ring_edges), in
the same length unit as the pitch."""
from __future__ import annotations

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
