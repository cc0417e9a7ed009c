"""Host-side FP64 setup physics of the plane solve: partial inductances, strip kernels and their spectra,
sheet impedances, the signal path's coupling into the strips, its own inductance and resistance.

These run once per geometry (kernels, coupling) or once per frequency (impedances) on the host; the
per-iteration work is in the CUDA library.  The formulas are GroundTruth's:

* filament mutual inductance (Neumann, closed form)      src/groundtruth/solver/kernel.py:165-176
* flat-tape mutual by the width-difference integral       src/groundtruth/solver/kernel.py:219-265
* strip self inductance (numeric) / GMD formula           src/groundtruth/solver/kernel.py:179-206
* narrow strips' self / side-by-side mutual changes      src/groundtruth/solver/peec.py:3309-3342
* strip kernel: filaments far, tapes for |offset| <= 4    src/groundtruth/solver/kernel.py:268-294
* one-face slab impedance, Dowell skin thickness          src/groundtruth/solver/kernel.py:23-75
* vector potential of a filament, segment mutual          src/groundtruth/solver/kernel.py:297-337
* strip coupling psi (3 x 3 Gauss points near the trace)  src/groundtruth/solver/peec.py:2615-2656
* trace self inductance and resistance                    src/groundtruth/solver/peec.py:3227-3250

The spectra are computed at this build's own padded FFT sizes (any size >= 2n - 1 gives the same linear
convolution; the reference uses scipy's next_fast_len, peec.py:1952-1953).
"""
from __future__ import annotations

from functools import lru_cache

import numpy as np
from numpy.polynomial import legendre

MU0 = 4e-7 * np.pi
GMD_FLAT = 0.2235
NEAR = 4                 # kernel.py:287: offsets integrated as tapes
PANELS, ORDER = 30, 8    # kernel.py:215-216


def round12(v: float) -> float:
    """A pitch or gap as the kernels are computed for it: 12 significant digits (peec.py:3264-3273)."""
    return float(f"{float(v):.12g}")


@lru_cache(maxsize=None)
def gauss(n: int):
    x, w = legendre.leggauss(n)
    return x, w


def filament_mutual(length, axial, rho):
    rho = np.maximum(rho, 1e-12 * length)

    def G(u):
        return u * np.arcsinh(u / rho) - np.sqrt(u * u + rho * rho)
    return MU0 / (4 * np.pi) * (G(axial + length) - 2 * G(axial) + G(axial - length))


def panel_rule(lo: float, hi: float, graded_end, panels: int, order: int):
    """Gauss-Legendre nodes and weights (order points per panel) over [lo, hi] cut into `panels` panels: equal
    ones, or, toward an integrable log singularity at graded_end (lo or hi), panels that halve in length so the
    one touching it is 2^-(panels - 1) of the interval."""
    x, w = gauss(order)
    if graded_end is None:
        edges = np.linspace(0.0, 1.0, panels + 1)
    else:
        edges = np.concatenate([[0.0], np.ldexp(1.0, np.arange(1 - panels, 1))])   # 0, 2^(1-p), ..., 1/2, 1
        if graded_end == hi:
            edges = 1.0 - edges[::-1]
    mid, half = 0.5 * (edges[1:] + edges[:-1]), 0.5 * (edges[1:] - edges[:-1])
    span = hi - lo
    nodes = lo + span * (mid[:, None] + half[:, None] * x[None, :])
    return nodes.ravel(), (span * half[:, None] * w[None, :]).ravel()


def tape_mutual(length, wa, wb, axial, lateral, dz) -> float:
    """Mutual inductance of two parallel flat tapes of one length, widths wa and wb, their centres `axial` apart
    along them, `lateral` across and dz out of plane: the mean filament mutual over all filament pairs,
    (1 / wa wb) int W(v) M(length, axial, |(lateral + v, dz)|) dv over the pairs' lateral separation v, W(v) the
    length of the widths' overlap at that separation (min(wa, wb) flat, falling to 0 at |v| = (wa + wb) / 2).
    The integral is cut at W's corners and at v = -lateral, where filaments line up (a log singularity when dz
    is 0): graded panels beside that point, four equal ones elsewhere."""
    reach, flat = 0.5 * (wa + wb), 0.5 * abs(wa - wb)
    sing = -lateral
    cuts = {-reach, -flat, flat, reach}
    if abs(sing) < reach:
        cuts.add(sing)
    cuts = sorted(cuts)
    nodes, weights = [], []
    for lo, hi in zip(cuts[:-1], cuts[1:]):
        if hi <= lo:
            continue
        end = lo if lo == sing else hi if hi == sing else None
        v, wt = panel_rule(lo, hi, end, PANELS if end is not None else 4, ORDER)
        nodes.append(v)
        weights.append(wt)
    v, wt = np.concatenate(nodes), np.concatenate(weights)
    overlap = np.clip(np.minimum(reach - np.abs(v), min(wa, wb)), 0.0, None)
    m = filament_mutual(length, np.full(len(v), float(axial)), np.hypot(lateral + v, dz))
    return float(np.dot(wt * overlap, m)) / (wa * wb)


def strip_self(length: float, width: float, thickness: float = 0.0) -> float:
    return float(filament_mutual(length, np.array(0.0), np.array(GMD_FLAT * (width + thickness))))


def strip_self_numeric(length: float, width):
    """A flat strip's partial self inductance as the mean filament mutual over its width pairs, by a graded
    Gauss rule toward the coincident pair (kernel.py:187-206).  width may be an array."""
    s, ws = panel_rule(0.0, 1.0, 0.0, PANELS, ORDER)
    w = np.atleast_1d(np.asarray(width, float)).ravel()
    u = w[:, None] * s[None, :]
    out = 2.0 * (filament_mutual(length, 0.0, u) * ((1.0 - s) * ws)[None, :]).sum(axis=1)
    return float(out[0]) if np.ndim(width) == 0 else out.reshape(np.shape(width))


NEAR_AXIAL = 2      # peec.py:3325: side-by-side partial strips corrected up to this many strips along


def narrow_self(d: float, phi, t):
    """The partial self inductance a strip d long and phi*d wide (copper t thick) adds to the full square
    strip's (peec.py:3309-3322): the numeric flat-strip integral's change and the GMD formula's thickness
    change."""
    phi, t = np.asarray(phi, float), np.asarray(t, float)

    def thick(w):
        return filament_mutual(d, 0.0, GMD_FLAT * w) - filament_mutual(d, 0.0, GMD_FLAT * (w + t))
    return strip_self_numeric(d, phi * d) - strip_self_numeric(d, d) - thick(phi * d) + thick(d)


def side_mutual(length: float, wa, wb, gap, steps=0.0, n: int = 8) -> np.ndarray:
    """Mutual inductance of two flat coplanar parallel strips, widths wa and wb, centres gap apart across them
    and `steps` lengths apart along them (fractions of `length`): the mean of n x n filament mutuals, touching
    filaments a filament's GMD apart (peec.py:3328-3341)."""
    wa, wb, gap, steps = (np.atleast_1d(v) for v in np.broadcast_arrays(*(np.asarray(v, float) for v in
                                                                            (wa, wb, gap, steps))))
    wa, wb, gap = wa * length, wb * length, gap * length
    u = (np.arange(n) + 0.5) / n - 0.5
    ya = wa[:, None, None] * u[None, :, None]
    yb = gap[:, None, None] + wb[:, None, None] * u[None, None, :]
    rho = np.maximum(np.abs(yb - ya), GMD_FLAT * np.maximum(wa, wb)[:, None, None] / n)
    axial = np.broadcast_to((steps * length)[:, None, None], rho.shape)
    return filament_mutual(length, axial, rho).mean(axis=(1, 2))


def near_values(n_axial: int, n_lateral: int, d: float, dz: float) -> np.ndarray:
    """(NEAR+1, NEAR+1) tape-integrated mutual inductances at the nearest offsets (kernel.py:287-294); offsets
    beyond the grid are zero."""
    out = np.zeros((NEAR + 1, NEAR + 1))
    for oa in range(min(NEAR, n_axial - 1) + 1):
        for ol in range(min(NEAR, n_lateral - 1) + 1):
            out[oa, ol] = tape_mutual(d, d, d, oa * d, ol * d, dz)
    return out


def strip_kernel(n_axial: int, n_lateral: int, d: float, dz: float) -> np.ndarray:
    """(2 n_axial - 1, 2 n_lateral - 1) mutual inductances of square strips (side d, dz apart out of plane) at
    every grid offset: filaments along the strips' axes, replaced by the tape integral (near_values) where
    both |offsets| are at most NEAR pitches; the block is even in both offsets."""
    axial = np.arange(1 - n_axial, n_axial) * d
    across = np.arange(1 - n_lateral, n_lateral) * d
    K = filament_mutual(d, axial[:, None], np.hypot(across[None, :], dz))
    na, nl = min(NEAR, n_axial - 1), min(NEAR, n_lateral - 1)
    near = near_values(n_axial, n_lateral, d, dz)
    K[n_axial - 1 - na: n_axial + na, n_lateral - 1 - nl: n_lateral + nl] = \
        near[np.ix_(np.abs(np.arange(-na, na + 1)), np.abs(np.arange(-nl, nl + 1)))]
    return K


def spectrum_quadrant(K: np.ndarray, P0: int, P1: int) -> np.ndarray:
    """Real (P0//2+1, P1//2+1) quadrant of the DFT of the centred even kernel wrapped onto a P0 x P1 torus."""
    Z = np.zeros((P0, P1))
    c0, c1 = K.shape[0] // 2, K.shape[1] // 2
    Z[: K.shape[0], : K.shape[1]] = K
    Z = np.roll(Z, (-c0, -c1), axis=(0, 1))
    return np.ascontiguousarray(np.fft.fft2(Z).real[: P0 // 2 + 1, : P1 // 2 + 1])


def skin_depth(f, sigma):
    """delta = 1 / sqrt(pi f mu0 sigma); infinite at f = 0."""
    with np.errstate(divide="ignore"):
        return 1.0 / np.sqrt(np.pi * np.asarray(f, float) * MU0 * sigma)


def _depths(t, f, sigma) -> np.ndarray:
    """x = t / delta, the copper's thickness in skin depths (0 at DC)."""
    t, f = np.broadcast_arrays(np.asarray(t, float), np.asarray(f, float))
    return np.where(f > 0, t * np.sqrt(np.pi * np.maximum(f, 1e-300) * MU0 * sigma), 0.0)


def u_coth_u(x) -> np.ndarray:
    """u coth u at u = (1 + j) x, x >= 0: the one-face slab's impedance in units of its DC resistance.  Below
    x = 0.1 its Laurent series to x^4 (u^2 = 2 j x^2, u^4 = -4 x^4): 1 + j 2 x^2 / 3 + 4 x^4 / 45; above, the
    closed form with coth u = (1 + e^-2u) / (1 - e^-2u), which needs no clamp for thick copper."""
    x = np.asarray(x, float)
    u = (1 + 1j) * x
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        e = np.exp(-2.0 * u)
        closed = u * (1.0 + e) / (1.0 - e)
    series = 1.0 + 4.0 * x ** 4 / 45.0 + 1j * (2.0 * x ** 2 / 3.0)
    return np.where(x < 0.1, series, closed)


def slab_impedance(t, f, sigma):
    """Internal impedance per square of a slab t thick whose current returns on one face (kernel.py:47-75):
    u coth u / (sigma t), u = (1 + j) t / delta."""
    out = u_coth_u(_depths(t, f, sigma)) / (sigma * np.asarray(t, float))
    return complex(out) if np.ndim(out) == 0 else out


def face_sheet_impedance(t, f, sigma):
    """(z_self, z_mutual) per square of a slab's two face sheets t apart with free space between them: the sum
    mode u coth(u/2) and the difference mode beside the free space u^2 tanh(u/2) / (u - 2 tanh(u/2)), in units of
    1/(sigma t), u = (1 + j) t / delta, thin foils (t / delta < 0.1) by their series (kernel.py:102-152)."""
    t = np.asarray(t, float)
    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        delta = 1.0 / np.sqrt(np.pi * max(f, 1e-300) * MU0 * sigma)
        x = t / delta if f > 0 else np.zeros_like(t)
        u = (1 + 1j) * x
        th = np.tanh(np.where(x > 0, (1 + 1j) * np.minimum(x, 60.0), 1.0) / 2)
        small = x < 0.1
        zs = np.where(small, 2.0 + x ** 4 / 90.0 + 1j * (x ** 2 / 3.0 - x ** 6 / 1890.0), u / th)
        zd = np.where(small, 6.0 + x ** 4 / 350.0 + 1j * x ** 2 / 5.0, u * u * th / (u - 2.0 * th))
    return 0.5 * (zs + zd) / (sigma * t), 0.5 * (zs - zd) / (sigma * t)


def skin_thickness(t, f, sigma):
    """The thickness a DC resistance takes to give the slab's AC resistance: t / Re(u coth u), since
    Re(u coth u) = x (sinh 2x + sin 2x) / (cosh 2x - cos 2x) is the one-face slab's resistance ratio."""
    out = np.asarray(t, float) / u_coth_u(_depths(t, f, sigma)).real
    return float(out) if np.ndim(out) == 0 else out


def vector_potential(a, b, pts, rho_min: float) -> np.ndarray:
    ab = b - a
    L = float(np.linalg.norm(ab))
    if L == 0:
        return np.zeros(len(pts))
    u = ab / L
    p = pts - a
    pu = p @ u
    rho = np.sqrt(np.maximum(np.einsum("ij,ij->i", p, p) - pu * pu, rho_min * rho_min))
    return MU0 / (4 * np.pi) * (np.arcsinh((L - pu) / rho) + np.arcsinh(pu / rho))


def segment_mutual(a1, b1, a2, b2, rho_min: float, n: int = 16) -> float:
    d2 = b2 - a2
    L2 = float(np.linalg.norm(d2))
    L1 = float(np.linalg.norm(b1 - a1))
    if L2 == 0 or L1 == 0:
        return 0.0
    x, w = gauss(n)
    pts = a2 + (0.5 * (x + 1))[:, None] * d2
    return float(np.dot((b1 - a1) / L1, d2 / L2) * 0.5 * L2 * np.sum(w * vector_potential(a1, b1, pts, rho_min)))


def _dist_to_segment(P, a, b):
    ab = b - a
    L2 = float(ab @ ab)
    if L2 == 0:
        return np.linalg.norm(P - a, axis=1)
    t = np.clip((P - a) @ ab / L2, 0, 1)
    return np.linalg.norm(P - (a + t[:, None] * ab), axis=1)


def strip_coupling(segments: np.ndarray, strips: list, d: float, zs: np.ndarray, ts: np.ndarray) -> list:
    """psi (flux per ampere of signal) along each strip of each orientation.

    segments: rows (ax, ay, az, bx, by, bz, width, i); strips: [(k, i, j) arrays of the x strips,
    of the y strips].  Returns [psi_x, psi_y]."""
    x, w = gauss(3)
    q = 0.5 * x
    W = np.outer(w, w).ravel() / 4.0
    qa, ql = (g.ravel() for g in np.meshgrid(q, q, indexing="ij"))
    horiz = [s for s in segments if np.linalg.norm(s[3:5] - s[0:2]) > 0]
    out = []
    for axis, idx in enumerate(strips):
        if len(idx) == 0:
            out.append(np.zeros(0))
            continue
        k, i, j = idx[:, 0], idx[:, 1], idx[:, 2]
        cen = np.stack([i * d + (d / 2 if axis == 0 else 0.0), j * d + (d / 2 if axis == 1 else 0.0), zs[k]], 1)
        acc = np.zeros(len(idx))
        half = 0.5 * ts[k]
        for s in horiz:
            a, b, width, cur = s[0:3], s[3:6], float(s[6]), float(s[7])
            ab = b - a
            L = float(np.linalg.norm(ab))
            if abs(ab[axis]) < 1e-15 * L:
                continue
            cen[:, 2] = zs[k] + np.where(0.5 * (a[2] + b[2]) > zs[k], half, -half)
            rmin = max(0.5 * width, 1e-7)
            ac = vector_potential(a, b, cen, rmin)
            near = _dist_to_segment(cen, a, b) < 3 * d + 2 * width
            if near.any():
                c = cen[near]
                da, dl = (qa, ql) if axis == 0 else (ql, qa)
                pts = np.stack([c[:, 0, None] + da * d, c[:, 1, None] + dl * d,
                                np.broadcast_to(c[:, 2, None], (len(c), len(W)))], 2)
                ac[near] = (vector_potential(a, b, pts.reshape(-1, 3), rmin).reshape(len(c), len(W)) * W).sum(1)
            acc += (cur * ab[axis] / L) * ac
        out.append(d * acc)
    return out


def trace_self(segments: np.ndarray, trace_t: float) -> float:
    segs = [s for s in segments if np.linalg.norm(s[3:6] - s[0:3]) > 0]
    L = 0.0
    for n, si in enumerate(segs):
        L += si[7] ** 2 * strip_self(float(np.linalg.norm(si[3:6] - si[0:3])), float(si[6]), trace_t)
        for sj in segs[n + 1:]:
            L += 2 * si[7] * sj[7] * segment_mutual(si[0:3], si[3:6], sj[0:3], sj[3:6], GMD_FLAT * (si[6] + trace_t))
    return float(L)


def trace_resistance(segments: np.ndarray, f: float, sigma: float, trace_t: float) -> float:
    R = 0.0
    for s in segments:
        L = float(np.linalg.norm(s[3:6] - s[0:3]))
        if L == 0 or abs(s[5] - s[2]) > 0:
            continue
        R += s[7] ** 2 * L / (sigma * s[6] * skin_thickness(trace_t, f, sigma))
    return R


def sheet_blocks(L_self: float, centre: np.ndarray, sums: np.ndarray) -> np.ndarray:
    """Per-position layer block with each pair's cavity inductance (peec.py:3344-3359)."""
    N = len(sums)
    D = np.maximum(2.0 * (sums[0, 0] - sums), 0.0)
    np.fill_diagonal(D, 0.0)
    beta = max((L_self + centre[k, l]) / 2 + D[k, l] / 4 for k in range(N) for l in range(N) if k != l)
    B = beta - D / 2
    for _ in range(60):
        if np.linalg.eigvalsh(B).min() > 0.05 * L_self:
            break
        B += 0.25 * L_self
    return B


def fft_size(m: int) -> int:
    """The padded FFT length this build uses for a linear convolution needing >= m points: the smallest
    2^a or 3 * 2^a (a >= 3) at least m (radix-2/4/8 stages plus at most one radix-3 stage)."""
    best = None
    for base in (1, 3):
        p = 8 * base
        while p < m:
            p *= 2
        best = p if best is None else min(best, p)
    return best
