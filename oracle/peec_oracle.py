"""CPU oracle for the quasi-static PEEC plane-current solve (test infrastructure only).

This module is the checker, never the product: only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it.  The shipped solve runs in the
CUDA library under ``groundtruth_gb300/`` and fails loudly when that library is missing.

It restates, in plain numpy/scipy FP64, the algorithm of GroundTruth's solver for the scope the GPU build
covers (one current sheet per layer, no face sheets):

* partial inductances and the strip kernel      src/groundtruth/solver/kernel.py:165-294
* slab impedance / skin thickness               src/groundtruth/solver/kernel.py:23-75
* kernel spectra                                src/groundtruth/solver/peec.py:3276-3306, 3362-3371
* topology, components, reference nodes         src/groundtruth/solver/peec.py:1596-1656, 1845-1862
* 'sheet' preconditioner blocks                 src/groundtruth/solver/peec.py:2032-2052, 3344-3359
* impedances, preconditioner admittance         src/groundtruth/solver/peec.py:2150-2178, 2465-2511
* Schur complement + sparse factor              src/groundtruth/solver/peec.py:2379, 2423 (SuperLU)
* system product / preconditioner               src/groundtruth/solver/peec.py:3043-3083
* restarted GMRES (CGS + DGKS, Givens)          src/groundtruth/solver/peec.py:3093-3224
* solve driver                                  src/groundtruth/solver/peec.py:2560-2607
* derived stacks (added branches, Woodbury)     src/groundtruth/solver/peec.py:1871-1923, 2354-2377
* strips narrower than the pitch (dL, M_near)   src/groundtruth/solver/peec.py:1732-1820, 2129-2132, 3309-3342
* excitation, coupling, moment, loop impedance  src/groundtruth/solver/peec.py:2615-2817, 3227-3250

Parity of this restatement is pinned by ``tests/golden/*.npz``, produced by the reference itself
(``tests/golden/make_golden.py``) and checked by ``tests/test_oracle_golden.py``.
"""
from __future__ import annotations

import copy
import math
from dataclasses import dataclass, field
from typing import Callable, Optional

import numpy as np
import scipy.sparse as sp
from numpy.polynomial import legendre
from scipy.fft import fft2, ifft2, next_fast_len
from scipy.linalg import solve_triangular
from scipy.sparse.csgraph import connected_components
from scipy.sparse.linalg import splu

MU0 = 4e-7 * np.pi
GMD_FLAT = 0.2235            # kernel.py:21
SIGMA_CU = 5.8e7             # peec.py:74
KERNEL_DIGITS = 12           # peec.py:3259
GMRES_EXTRA_CYCLES = 24      # peec.py:98
GMRES_PROGRESS = 0.7         # peec.py:99
GMRES_CHECK_MISSES = 4       # peec.py:100
LU_PIVOT_THRESHOLD = 0.1     # peec.py:105
# FFT threads of the L_p product: all host cores (-1), as the reference's fft_workers() defaults (peec.py:136-149,
# a per-thread setting there); a process that solves alongside others on the same host sets it to 1
FFT_WORKERS = -1
TAPE_PANELS, TAPE_ORDER = 30, 8   # kernel.py:215-216


class OracleSolverError(RuntimeError):
    """The oracle's counterpart of peec.SolverError (peec.py:124)."""


# ----------------------------------------------------------------------------------------------- kernel.py
def cache_value(v: float) -> float:
    """v to 12 significant digits (peec.py:3264-3267)."""
    return float(f"{float(v):.{KERNEL_DIGITS}g}")


def skin_thickness(t, f, sigma):
    """Dowell's one-sided slab effective thickness (kernel.py:23-44)."""
    t = np.asarray(t, float)
    f = np.asarray(f, float)
    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        delta = 1.0 / np.sqrt(np.pi * np.maximum(f, 1e-300) * MU0 * sigma)
        x = np.where(f > 0, t / delta, 0.0)
        y = np.minimum(2 * x, 60.0)
        exact = x * (np.sinh(y) + np.sin(y)) / (np.cosh(y) - np.cos(y))
        factor = np.where(x < 0.1, 1.0 + 4.0 * x ** 4 / 45.0, exact)
    out = t / factor
    return float(out) if out.ndim == 0 else out


def slab_impedance(t, f, sigma):
    """(1+j)/(sigma delta) coth((1+j) t/delta) with the thin-foil series (kernel.py:47-75)."""
    t = np.asarray(t, float)
    f = np.asarray(f, float)
    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        delta = 1.0 / np.sqrt(np.pi * np.maximum(f, 1e-300) * MU0 * sigma)
        x = np.where(f > 0, t / delta, 0.0)
        u = (1 + 1j) * np.minimum(x, 30.0)
        exact = (1 + 1j) * x / np.tanh(np.where(x > 0, u, 1.0))
        series = 1.0 + 4.0 * x ** 4 / 45.0 + 1j * (2.0 * x ** 2 / 3.0)
        factor = np.where(x < 0.1, series, exact)
    out = factor / (sigma * t)
    return complex(out) if out.ndim == 0 else out


_LEG: dict = {}


def leggauss(n: int):
    """Gauss-Legendre nodes/weights (kernel.py:137-145)."""
    if n not in _LEG:
        _LEG[n] = legendre.leggauss(n)
    return _LEG[n]


def _antideriv(u, rho):
    """u asinh(u/rho) - sqrt(u^2+rho^2) (kernel.py:165-167)."""
    return u * np.arcsinh(u / rho) - np.sqrt(u * u + rho * rho)


def filament_mutual(length, axial, rho):
    """Parallel equal filaments, Neumann integral in closed form (kernel.py:170-176)."""
    rho = np.maximum(rho, 1e-12 * length)
    return MU0 / (4 * np.pi) * (_antideriv(axial + length, rho) - 2 * _antideriv(axial, rho)
                                + _antideriv(axial - length, rho))


def strip_self(length: float, width: float, thickness: float = 0.0) -> float:
    """Filament formula at the flat strip's GMD (kernel.py:179-184)."""
    return float(filament_mutual(length, np.array(0.0), np.array(GMD_FLAT * (width + thickness))))


def panel_rule(p: float, q: float, toward, panels: int, order: int):
    """Composite Gauss-Legendre rule, optionally graded geometrically toward one end (kernel.py:219-236)."""
    x, w = leggauss(order)
    if toward is None:
        edges = np.linspace(0.0, 1.0, panels + 1)
    else:
        edges = np.concatenate([[0.0], 0.5 ** np.arange(panels - 1, -1, -1)])
        if toward == q:
            edges = 1.0 - edges[::-1]
    lo, hi = edges[:-1], edges[1:]
    nodes = p + (q - p) * (lo[:, None] + (hi - lo)[:, None] * (x[None, :] + 1.0) / 2.0)
    weights = (q - p) * (hi - lo)[:, None] * w[None, :] / 2.0
    return nodes.ravel(), weights.ravel()


def strip_self_numeric(length: float, width):
    """Mean filament mutual over a flat strip's width pairs (kernel.py:187-206)."""
    s, ws = panel_rule(0.0, 1.0, 0.0, TAPE_PANELS, TAPE_ORDER)
    w = np.atleast_1d(np.asarray(width, float)).ravel()
    u = w[:, None] * s[None, :]
    out = 2.0 * (filament_mutual(length, 0.0, u) * ((1.0 - s) * ws)[None, :]).sum(axis=1)
    return float(out[0]) if np.ndim(width) == 0 else out.reshape(np.shape(width))


def tape_mutual(length, wa, wb, axial, lateral, dz) -> float:
    """Two parallel flat tapes: the width-difference integral split at the trapezoid's bends and at the
    filaments' crossing point (kernel.py:239-265)."""
    h, k, s = 0.5 * (wa + wb), 0.5 * abs(wa - wb), -lateral
    cuts = {-h, -k, k, h}
    if -h < s < h:
        cuts.add(s)
    pts = sorted(cuts)
    total = 0.0
    for p, q in zip(pts[:-1], pts[1:]):
        if q - p <= 0.0:
            continue
        toward = p if p == s else q if q == s else None
        v, wt = panel_rule(p, q, toward, TAPE_PANELS if toward is not None else 4, TAPE_ORDER)
        W = np.clip(np.minimum(0.5 * wa, v + 0.5 * wb) - np.maximum(-0.5 * wa, v - 0.5 * wb), 0.0, None)
        rho = np.sqrt((lateral + v) ** 2 + dz * dz)
        total += float(np.sum(wt * W * filament_mutual(length, np.full(len(v), axial), rho)))
    return total / (wa * wb)


def strip_kernel(n_axial: int, n_lateral: int, d: float, dz: float = 0.0) -> np.ndarray:
    """Square-strip mutual inductance for every grid offset: filaments far, tapes for |offsets| <= 4
    (kernel.py:268-294)."""
    ia = np.arange(-(n_axial - 1), n_axial) * d
    il = np.arange(-(n_lateral - 1), n_lateral) * d
    A, L = np.meshgrid(ia, il, indexing="ij")
    K = filament_mutual(d, A, np.sqrt(L * L + dz * dz))
    ca, cl = n_axial - 1, n_lateral - 1
    for oa in range(0, min(4, n_axial - 1) + 1):
        for ol in range(0, min(4, n_lateral - 1) + 1):
            m = tape_mutual(d, d, d, oa * d, ol * d, dz)
            for pa in {ca + oa, ca - oa}:
                for pl in {cl + ol, cl - ol}:
                    K[pa, pl] = m
    return K


def kernel_spectrum(K: np.ndarray, P) -> np.ndarray:
    """Real quadrant of the FFT of the centred kernel embedded circularly in P (peec.py:3362-3371)."""
    Z = np.zeros(P)
    Z[: K.shape[0], : K.shape[1]] = K
    Z = np.roll(Z, (-(K.shape[0] // 2), -(K.shape[1] // 2)), axis=(0, 1))
    return np.ascontiguousarray(fft2(Z).real[: P[0] // 2 + 1, : P[1] // 2 + 1])


def kernel_pair(nx: int, ny: int, d: float, dz: float):
    """(x spectrum quadrant, y spectrum quadrant, centre, sum x, sum y) for one layer gap
    (peec.py:3276-3306; d and dz rounded to 12 digits first)."""
    d, dz = cache_value(d), cache_value(dz)
    Px = (next_fast_len(2 * (nx - 1) - 1), next_fast_len(2 * ny - 1))
    Py = (next_fast_len(2 * nx - 1), next_fast_len(2 * (ny - 1) - 1))
    kx = strip_kernel(nx - 1, ny, d, dz)
    ky = strip_kernel(ny - 1, nx, d, dz).T
    return (kernel_spectrum(kx, Px), kernel_spectrum(ky, Py), float(kx[nx - 2, ny - 1]), float(kx.sum()),
            float(ky.sum()), kx, ky)


def segment_vector_potential(a, b, points, rho_min: float = 1e-9) -> np.ndarray:
    """|A| per ampere of a straight filament at points (kernel.py:297-312)."""
    ab = b - a
    L = np.linalg.norm(ab)
    if L == 0:
        return np.zeros(len(points))
    u = ab / L
    p = points - a
    pu = p @ u
    rho2 = np.einsum("ij,ij->i", p, p) - pu * pu
    rho = np.sqrt(np.maximum(rho2, rho_min * rho_min))
    return MU0 / (4 * np.pi) * (np.arcsinh((L - pu) / rho) + np.arcsinh(pu / rho))


def segment_mutual(a1, b1, a2, b2, rho_min: float, n: int = 16) -> float:
    """Neumann mutual of two filaments, Gauss rule on the second (kernel.py:315-337)."""
    a2, b2 = np.asarray(a2, float), np.asarray(b2, float)
    d2 = b2 - a2
    L2 = np.linalg.norm(d2)
    if L2 == 0:
        return 0.0
    x, w = leggauss(n)
    t = 0.5 * (x + 1)
    pts = a2 + t[:, None] * d2
    a1, b1 = np.asarray(a1, float), np.asarray(b1, float)
    L1 = np.linalg.norm(b1 - a1)
    if L1 == 0:
        return 0.0
    psi = segment_vector_potential(a1, b1, pts, rho_min)
    return float(np.dot((b1 - a1) / L1, d2 / L2) * 0.5 * L2 * np.sum(w * psi))


def dist_to_segment(P, a, b):
    """Distance of points to a segment (peec.py:3374-3382)."""
    ab = b - a
    L2 = float(ab @ ab)
    if L2 == 0:
        return np.linalg.norm(P - a, axis=1)
    t = np.clip((P - a) @ ab / L2, 0, 1)
    return np.linalg.norm(P - (a + t[:, None] * ab), axis=1)


def sheet_blocks(L_self: float, centre: np.ndarray, sums: np.ndarray) -> np.ndarray:
    """Per-position layer block keeping each pair's cavity inductance (peec.py:3344-3359)."""
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


# ----------------------------------------------------------------------------------------------- GMRES
def gmres(op: Callable, b: np.ndarray, tol: float, max_cycles: int = 8, restart: int = 200,
          bnorm: Optional[float] = None, max_its: Optional[int] = None, extra_cycles: int = 0):
    """Restarted GMRES with CGS + DGKS re-orthogonalisation, Givens-triangular Hessenberg, true-residual
    check and stop (peec.py:3093-3224), complex128 basis."""
    n = len(b)
    if bnorm is None:
        bnorm = float(np.linalg.norm(b))
    x = np.zeros(n, complex)
    if bnorm == 0 or np.linalg.norm(b) <= tol * bnorm:
        return x, 0, True
    its = 0
    r = b.astype(complex)
    last = math.inf
    V = np.empty((restart + 1, n), complex)
    for cycle in range(max_cycles + extra_cycles):
        beta = float(np.linalg.norm(r))
        if beta <= tol * bnorm:
            return x, its, True
        if max_its is not None and its >= max_its:
            return x, its, False
        if cycle >= max_cycles and beta > GMRES_PROGRESS * last:
            return x, its, False
        last = beta
        H = np.zeros((restart + 1, restart), complex)
        cs = np.zeros(restart)
        sn = np.zeros(restart, complex)
        g = np.zeros(restart + 1, complex)
        g[0] = beta
        V[0] = r / beta
        k = 0
        aim = tol * bnorm
        misses = 0
        restarted = False
        for j in range(restart):
            w = op(V[j])
            w_norm = float(np.linalg.norm(w))
            h = V[: j + 1].conj() @ w
            w = w - V[: j + 1].T @ h
            hn = float(np.linalg.norm(w))
            if hn < 0.7 * w_norm:
                h2 = V[: j + 1].conj() @ w
                w = w - V[: j + 1].T @ h2
                h = h + h2
                hn = float(np.linalg.norm(w))
            col = np.empty(j + 2, complex)
            col[: j + 1] = h
            col[j + 1] = hn
            for i in range(j):
                a, c = col[i], col[i + 1]
                col[i] = cs[i] * a + sn[i] * c
                col[i + 1] = -np.conj(sn[i]) * a + cs[i] * c
            a = col[j]
            rho = math.hypot(abs(a), hn)
            if rho == 0.0:
                cs[j], sn[j] = 1.0, 0.0
            elif abs(a) == 0.0:
                cs[j], sn[j] = 0.0, 1.0
                col[j] = hn
            else:
                phase = a / abs(a)
                cs[j], sn[j] = abs(a) / rho, phase * hn / rho
                col[j] = phase * rho
            col[j + 1] = 0.0
            H[: j + 2, j] = col
            g[j + 1] = -np.conj(sn[j]) * g[j]
            g[j] = cs[j] * g[j]
            its += 1
            k = j + 1
            if hn <= 1e-14 * np.linalg.norm(h) or (max_its is not None and its >= max_its):
                break
            if abs(g[j + 1]) <= aim:
                y = solve_triangular(H[:k, :k], g[:k])
                xt = x + y @ V[:k]
                rt = b - op(xt)
                if np.linalg.norm(rt) <= tol * bnorm:
                    return xt, its, True
                misses += 1
                if misses >= GMRES_CHECK_MISSES:
                    x, r = xt, rt
                    restarted = True
                    break
                aim = 0.5 * abs(g[j + 1])
            V[j + 1] = w / hn
        if restarted:
            continue
        while k and H[k - 1, k - 1] == 0:
            k -= 1
        y = solve_triangular(H[:k, :k], g[:k]) if k else np.zeros(0, complex)
        x = x + y @ V[:k]
        r = b - op(x)
    return x, its, bool(np.linalg.norm(r) <= tol * bnorm)


SCREEN_MIN_NODES = 16   # peec.py: a layer with this many nodes under copper above and below is split into faces


def slab_modes(t, f, sigma, free_space: bool = False):
    """(zs, zd) of a slab t thick in units of 1/(sigma t): u coth(u/2) and u tanh(u/2), u = (1 + j) t / delta; with
    free_space the difference mode beside the free space between two face sheets, u^2 tanh(u/2) / (u - 2 tanh(u/2));
    thin foils (t / delta < 0.1) by their series (kernel.py:130-152)."""
    t = np.asarray(t, float)
    f = np.asarray(f, float)
    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        delta = 1.0 / np.sqrt(np.pi * np.maximum(f, 1e-300) * MU0 * sigma)
        x = np.where(f > 0, t / delta, 0.0)
        u = (1 + 1j) * x
        th = np.tanh(np.where(x > 0, (1 + 1j) * np.minimum(x, 60.0), 1.0) / 2)
        small = x < 0.1
        zs = np.where(small, 2.0 + x ** 4 / 90.0 + 1j * (x ** 2 / 3.0 - x ** 6 / 1890.0), u / th)
        if free_space:
            zd = np.where(small, 6.0 + x ** 4 / 350.0 + 1j * x ** 2 / 5.0, u * u * th / (u - 2.0 * th))
        else:
            zd = np.where(small, x ** 4 / 6.0 + 1j * (x ** 2 - x ** 6 / 30.0), u * th)
    return zs, zd


def face_sheet_impedance(t, f, sigma):
    """(z_self, z_mutual) per square of a slab's two face sheets t apart with free space between them
    (kernel.py:102-127)."""
    t = np.asarray(t, float)
    zs, zdm = slab_modes(t, f, sigma, free_space=True)
    return 0.5 * (zs + zdm) / (sigma * t), 0.5 * (zs - zdm) / (sigma * t)


NEAR_AXIAL = 2      # peec.py:3325: side-by-side partial strips corrected up to this many strips along


def narrow_self(d: float, phi, t):
    """The partial self inductance a strip d long and phi*d wide adds to the full square strip's: the numeric
    flat-strip integral's change plus the thickness change of the GMD formula (peec.py:3309-3322)."""
    phi, t = np.asarray(phi, float), np.asarray(t, float)

    def thick(w):
        return filament_mutual(d, 0.0, GMD_FLAT * w) - filament_mutual(d, 0.0, GMD_FLAT * (w + t))
    return strip_self_numeric(d, phi * d) - strip_self_numeric(d, d) - thick(phi * d) + thick(d)


def side_mutual(length: float, wa, wb, gap, steps=0.0, n: int = 8) -> np.ndarray:
    """Mutual inductance of two flat coplanar parallel strips (widths wa, wb, centre distance gap, `steps`
    lengths apart along them; fractions of `length`): the mean of n x n filament mutuals, touching filaments a
    filament's GMD apart (peec.py:3328-3341)."""
    wa, wb, gap, steps = (np.atleast_1d(v) for v in np.broadcast_arrays(*(np.asarray(v, float) for v in
                                                                            (wa, wb, gap, steps))))
    wa, wb, gap = wa * length, wb * length, gap * length
    u = (np.arange(n) + 0.5) / n - 0.5
    ya = wa[:, None, None] * u[None, :, None]
    yb = gap[:, None, None] + wb[:, None, None] * u[None, None, :]
    rho = np.maximum(np.abs(yb - ya), GMD_FLAT * np.maximum(wa, wb)[:, None, None] / n)
    axial = np.broadcast_to((steps * length)[:, None, None], rho.shape)
    return filament_mutual(length, axial, rho).mean(axis=(1, 2))


# ----------------------------------------------------------------------------------------------- problem
@dataclass
class OLayer:
    """One plane layer: height z (m), copper thickness (m), node / strip masks on the shared grid."""
    z: float
    thickness: float
    node: np.ndarray
    xb: np.ndarray
    yb: np.ndarray
    widths: Optional[dict] = None     # the grid's wx / wy, ox / oy, rx / ry (peec.py:213-220); None: full strips
    fill: Optional[np.ndarray] = None  # the grid's cells' copper fraction (peec.py:211); None: the node mask


@dataclass
class OPair:
    """Plane-pair capacitance between two layers (peec.py:1041-1048)."""
    upper: int
    lower: int
    c_per_area: float
    tan_delta: float = 0.02


@dataclass
class OBranch:
    """A lumped branch between two (layer, i, j) nodes with impedance R + jwL (+ 1/(jwC) when C > 0)."""
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
class OSegment:
    """A straight piece of the known current path (peec.py:1051-1058)."""
    a: np.ndarray
    b: np.ndarray
    width: float
    i: float = 1.0


class OracleStack:
    """Everything of peec.PlaneStack the scope needs: topology, kernels, per-frequency operators, products."""

    def __init__(self, layers: list, d: float, branches=None, pairs=None, sigma: float = SIGMA_CU,
                 precond: str = "diag", screen: bool = False):
        if precond not in ("diag", "sheet"):
            raise ValueError("precond must be 'diag' or 'sheet'")
        self.layers = list(layers)
        self.N = len(layers)
        self.nx, self.ny = layers[0].node.shape
        self.d = d                                       # metres
        self.zs = np.array([l.z for l in layers], float)
        self.sigma = sigma
        self.pairs = list(pairs or [])
        self.precond_mode = precond
        self.screen = screen
        self.layer_t = np.array([l.thickness for l in layers], float)
        self._base: Optional[OracleStack] = None
        self.r_scale = self.branch_scale = None
        self._topology(list(branches or []))
        self._kernels()
        self._widths()

    # -- face sheets of screened layers (peec.py:1658-1723)
    def _faces(self, node: np.ndarray):
        """twin_parent, n_sheets, sheet_layer, sheet_z, sheet_t (peec.py:1658-1697)."""
        N = self.N
        t = self.layer_t
        twins = []
        if self.screen and N >= 3:
            for k in range(N):
                above = np.zeros(node.shape[1:], bool)
                below = np.zeros(node.shape[1:], bool)
                for m in range(N):
                    if self.zs[m] > self.zs[k]:
                        above |= node[m]
                    elif self.zs[m] < self.zs[k]:
                        below |= node[m]
                if int(np.count_nonzero(node[k] & above & below)) >= SCREEN_MIN_NODES:
                    twins.append(k)
        self.twin_parent = np.array(twins, np.int64)
        self.n_sheets = N + len(twins)
        self.sheet_layer = np.concatenate([np.arange(N), self.twin_parent]).astype(np.int64)
        z = self.zs.copy()
        st = t.copy()
        z[twins] = self.zs[twins] + 0.5 * t[twins]
        st[twins] = 0.0
        self.sheet_z = np.concatenate([z, self.zs[twins] - 0.5 * t[twins]])
        self.sheet_t = np.concatenate([st, np.zeros(len(twins))])

    def _twins(self):
        """tw_a / tw_b: each split layer's upper-face strips and the twin's (peec.py:1699-1716)."""
        N = self.N
        a, b = [], []
        for xb, lo in ((self.xb, 0), (self.yb, self.nxb)):
            per = np.count_nonzero(xb.reshape(self.n_sheets, -1), axis=1)
            start = lo + np.concatenate([[0], np.cumsum(per)[:-1]])
            for m, p in enumerate(self.twin_parent):
                a.append(start[p] + np.arange(per[p]))
                b.append(start[N + m] + np.arange(per[p]))
        self.tw_a = np.concatenate(a).astype(np.int64) if a else np.zeros(0, np.int64)
        self.tw_b = np.concatenate(b).astype(np.int64) if b else np.zeros(0, np.int64)

    def layer_index(self, orient: str) -> np.ndarray:
        """The orientation's strips as (layer, i, j) rows (peec.py:1718-1729)."""
        idx = (self.xa if orient == "x" else self.ya).copy()
        idx[:, 0] = self.sheet_layer[idx[:, 0]]
        return idx

    def sheet_of_strip(self, strips: np.ndarray) -> np.ndarray:
        strips = np.asarray(strips, np.int64)
        out = np.empty(len(strips), np.int64)
        x = strips < self.nxb
        out[x] = self.xa[strips[x], 0]
        out[~x] = self.ya[strips[~x] - self.nxb, 0]
        return out

    # -- strips narrower than the pitch (peec.py:1732-1820, 3309-3342)
    def _widths(self):
        """strip_width, r_width (ns), dL (ns or None) and M_near (sparse ns x ns or None): peec.py:1732-1820."""
        def gather(key, idx, shape, default):
            if len(idx) == 0:
                return np.zeros(0)
            if all((l.widths or {}).get(key) is None for l in self.layers):
                return np.full(len(idx), default)
            w = np.stack([np.asarray(l.widths[key], float) if (l.widths or {}).get(key) is not None
                          else np.full(shape, default) for l in self.layers])
            return w[tuple(idx.T)]
        sx, sy = (self.nx - 1, self.ny), (self.nx, self.ny - 1)
        lx, ly = self.layer_index("x"), self.layer_index("y")
        w = np.concatenate([gather("wx", lx, sx, 1.0), gather("wy", ly, sy, 1.0)])
        ok = w > 0
        self.strip_width = np.where(ok, w, 1.0)
        rw = np.concatenate([gather("rx", lx, sx, 0.0), gather("ry", ly, sy, 0.0)])
        self.r_width = np.where(ok & (rw > 0), rw, self.strip_width)
        self.r_uniform = not np.any(self.r_width != 1.0)
        off = np.where(ok, np.concatenate([gather("ox", lx, sx, 0.0), gather("oy", ly, sy, 0.0)]), 0.0)
        self.dL = self.M_near = None
        narrow = self.strip_width < 1.0
        if not np.any(narrow):
            return
        d = self.d
        t = self.layer_t[np.concatenate([lx[:, 0], ly[:, 0]])]
        dL = np.zeros(self.ns)
        keys, inv = np.unique(np.round(np.column_stack([self.strip_width[narrow], t[narrow]]), 12), axis=0,
                              return_inverse=True)
        dL[narrow] = narrow_self(d, keys[:, 0], keys[:, 1])[np.ravel(inv)]
        self.dL = dL
        rows, cols, steps = [], [], []
        for idx, shape, lo, axis in ((self.xa, sx, 0, 2), (self.ya, sy, self.nxb, 1)):
            if len(idx) == 0:
                continue
            at = -np.ones((self.n_sheets, *shape), np.int64)
            at[tuple(idx.T)] = lo + np.arange(len(idx))
            n_ax = shape[0] if axis == 2 else shape[1]
            for k in range(-NEAR_AXIAL, NEAR_AXIAL + 1):
                if abs(k) >= n_ax:
                    continue
                ax_a = slice(max(-k, 0), n_ax - max(k, 0))
                ax_b = slice(max(k, 0), n_ax - max(-k, 0))
                a = at[:, ax_a, :-1] if axis == 2 else at[:, :-1, ax_a]
                b = at[:, ax_b, 1:] if axis == 2 else at[:, 1:, ax_b]
                both = (a >= 0) & (b >= 0)
                a, b = a[both], b[both]
                part = narrow[a] | narrow[b]
                rows.append(a[part])
                cols.append(b[part])
                steps.append(np.full(int(part.sum()), abs(k)))
        a, b = np.concatenate(rows), np.concatenate(cols)
        if len(a) == 0:
            self._twin_corrections()
            return
        k = np.concatenate(steps)
        wa, wb = self.strip_width[a], self.strip_width[b]
        gap = 1.0 + off[b] - off[a]
        keys, inv = np.unique(np.round(np.column_stack([wa, wb, gap, k]), 9), axis=0, return_inverse=True)
        ones = np.ones(len(keys))
        dM = (side_mutual(d, keys[:, 0], keys[:, 1], keys[:, 2], keys[:, 3])
              - side_mutual(d, ones, ones, ones, keys[:, 3]))[np.ravel(inv)]
        M = sp.coo_matrix((dM, (a, b)), shape=(self.ns, self.ns))
        self.M_near = (M + M.T).tocsr()
        self._twin_corrections()

    def _twin_corrections(self):
        """A split layer's faces share their copper's narrow-width corrections (peec.py:1822-1843)."""
        if self.dL is None or not len(self.tw_b):
            return
        n = self.ns
        pairs = np.concatenate([self.tw_a, self.tw_b]), np.concatenate([self.tw_b, self.tw_a])
        extra = sp.coo_matrix((np.concatenate([self.dL[self.tw_a], self.dL[self.tw_b]]), pairs), shape=(n, n))
        if self.M_near is not None:
            swap = sp.coo_matrix((np.ones(len(pairs[0])), pairs), shape=(n, n)).tocsr()
            extra = extra + self.M_near @ swap
        self.M_near = ((self.M_near if self.M_near is not None else 0) + extra).tocsr()

    def with_branches(self, extra: list) -> "OracleStack":
        """This stack plus a few branches (peec.py:1871-1912): a shallow copy sharing the grids and kernels with
        its own incidence; its operators update the base's factorisation (operator below).  A branch joining
        two pieces of copper: a stack of its own."""
        extra = [b for b in extra if self.nid[b.a] >= 0 and self.nid[b.b] >= 0 and b.a != b.b]
        if not extra:
            return self
        a = np.array([self.nid[b.a] for b in extra])
        b = np.array([self.nid[b.b] for b in extra])
        if np.any(self.full_label[a] != self.full_label[b]):
            return OracleStack(self.layers, self.d, self.branches + extra, self.pairs, self.sigma, self.precond_mode)
        new = copy.copy(self)
        new._topology(self.branches + extra)
        new._base = self
        return new

    def map_state(self, x: Optional[np.ndarray], stack: "OracleStack") -> Optional[np.ndarray]:
        """A solution of the base in this stack's unknowns, the added branches at zero (peec.py:1914-1923)."""
        if x is None:
            return None
        if stack is self:
            return x
        if self._base is stack and len(x) == stack.nb + stack.Ar.shape[1]:
            return np.concatenate([x[: stack.nb], np.zeros(self.nb - stack.nb, complex), x[stack.nb:]])
        return None

    # -- topology (peec.py:1596-1656, 1845-1862)
    def _topology(self, branches):
        node = np.stack([l.node for l in self.layers])
        self.node = node
        xb = np.stack([l.xb for l in self.layers]) & node[:, :-1, :] & node[:, 1:, :]
        yb = np.stack([l.yb for l in self.layers]) & node[:, :, :-1] & node[:, :, 1:]
        self._faces(node)
        self.xb = np.concatenate([xb, xb[self.twin_parent]]) if len(self.twin_parent) else xb
        self.yb = np.concatenate([yb, yb[self.twin_parent]]) if len(self.twin_parent) else yb
        self.nid = -np.ones(node.shape, np.int64)
        idx = np.nonzero(node)
        self.nid[idx] = np.arange(len(idx[0]))
        self.n_nodes = self.n_grid = len(idx[0])
        self.xa, self.ya = np.argwhere(self.xb), np.argwhere(self.yb)
        self.nxb, self.nyb = len(self.xa), len(self.ya)
        self.ns = self.nxb + self.nyb
        self._twins()
        # a plane pair's capacitance per cell where both planes have copper and no layer between them does, over
        # the facing copper area of the cell (peec.py:1622-1637)
        cap = []
        cell = self.d ** 2
        fill = [l.fill if l.fill is not None else node[k].astype(float) for k, l in enumerate(self.layers)]
        for p in self.pairs:
            between = np.zeros(node.shape[1:], bool)
            for m in range(p.upper + 1, p.lower):
                between |= node[m]
            share = np.minimum(fill[p.upper], fill[p.lower])
            ii, jj = np.nonzero(node[p.upper] & node[p.lower] & ~between & (share > 0))
            cap.append(np.column_stack([np.full(len(ii), p.upper), np.full(len(ii), p.lower), ii, jj,
                                        p.c_per_area * cell * share[ii, jj], np.full(len(ii), p.tan_delta)]))
        self.cap = np.concatenate(cap) if cap else np.zeros((0, 6))
        self.ncap = len(self.cap)
        self.branches = [b for b in branches if self.nid[b.a] >= 0 and self.nid[b.b] >= 0 and b.a != b.b]
        self.nbr = len(self.branches)
        self.nb = self.ns + self.ncap + self.nbr
        cu = self.cap[:, :4].astype(np.int64)
        xa, ya = self.layer_index("x"), self.layer_index("y")       # a strip joins its layer's nodes
        self.a_nodes = np.concatenate([self.nid[tuple(xa.T)], self.nid[tuple(ya.T)], self.nid[cu[:, 0], cu[:, 2], cu[:, 3]],
                                       np.array([self.nid[b.a] for b in self.branches], np.int64)]).astype(np.int64)
        self.b_nodes = np.concatenate([self.nid[xa[:, 0], xa[:, 1] + 1, xa[:, 2]], self.nid[ya[:, 0], ya[:, 1], ya[:, 2] + 1],
                                       self.nid[cu[:, 1], cu[:, 2], cu[:, 3]],
                                       np.array([self.nid[b.b] for b in self.branches], np.int64)]).astype(np.int64)
        r = np.arange(self.nb)
        self.A = sp.csr_matrix((np.concatenate([np.ones(self.nb), -np.ones(self.nb)]),
                                (np.concatenate([r, r]), np.concatenate([self.a_nodes, self.b_nodes]))),
                               shape=(self.nb, self.n_nodes))
        n = self.n_nodes
        cond = np.ones(self.nb, bool)
        cond[self.ns: self.ns + self.ncap] = False
        g = sp.coo_matrix((np.ones(cond.sum()), (self.a_nodes[cond], self.b_nodes[cond])), shape=(n, n))
        _, self.cond_label = connected_components(g, directed=False)
        g = sp.coo_matrix((np.ones(self.nb), (self.a_nodes, self.b_nodes)), shape=(n, n))
        _, self.full_label = connected_components(g, directed=False)
        _, first = np.unique(self.full_label, return_index=True)
        self.keep = np.ones(n, bool)
        self.keep[first] = False
        self.Ar = self.A[:, self.keep].tocsc()
        self.ArT = self.Ar.T.tocsr()

    def face_gap(self, s: int, t: int) -> float:
        """The distance between the faces sheets s and t turn to each other (peec.py:1926-1933)."""
        if s == t:
            return 0.0
        return max(abs(self.sheet_z[s] - self.sheet_z[t]) - 0.5 * (self.sheet_t[s] + self.sheet_t[t]), 1e-6)

    # -- kernels (peec.py:1941-1988)
    def _kernels(self):
        """Spectra for every sheet pair, the self term and the 'sheet' blocks (peec.py:1941-2028)."""
        nx, ny, d, N = self.nx, self.ny, self.d, self.n_sheets
        self.Px = (next_fast_len(2 * (nx - 1) - 1), next_fast_len(2 * ny - 1))
        self.Py = (next_fast_len(2 * nx - 1), next_fast_len(2 * (ny - 1) - 1))
        Kx = np.empty((self.Px[0] // 2 + 1, self.Px[1] // 2 + 1, N, N))
        Ky = np.empty((self.Py[0] // 2 + 1, self.Py[1] // 2 + 1, N, N))
        self.L_self = kernel_pair(nx, ny, d, 0.0)[2]
        centre, sum_x, sum_y = np.zeros((N, N)), np.zeros((N, N)), np.zeros((N, N))
        self.kx_real, self.ky_real = {}, {}
        for s in range(N):
            for t in range(s, N):
                kx, ky, c, sx, sy, rx, ry = kernel_pair(nx, ny, d, self.face_gap(s, t))
                Kx[:, :, s, t] = Kx[:, :, t, s] = kx
                Ky[:, :, s, t] = Ky[:, :, t, s] = ky
                centre[s, t] = centre[t, s] = c
                sum_x[s, t] = sum_x[t, s] = sx
                sum_y[s, t] = sum_y[t, s] = sy
                self.kx_real[(s, t)] = rx
                self.ky_real[(s, t)] = ry
        self.Kq = {"x": Kx, "y": Ky}
        self.centre, self.sum_x, self.sum_y = centre, sum_x, sum_y
        self.blocks = []
        if self.precond_mode == "sheet" and self.N > 1:
            self.B_x = self._sheet_block(centre, sum_x)
            self.B_y = self._sheet_block(centre, sum_y)
            self._block_layout()
        elif len(self.twin_parent):
            # 'diag' with split layers: each face pair at a position is a 2 x 2 block (peec.py:1979-1987)
            B = np.diag(np.full(N, self.L_self))
            for m, p in enumerate(self.twin_parent):
                B[p, self.N + m] = B[self.N + m, p] = centre[p, self.N + m]
            self.B_x = self.B_y = B
            self._twin_blocks()

    def _sheet_block(self, centre: np.ndarray, sums: np.ndarray) -> np.ndarray:
        """'sheet' blocks made over the layers, a split layer's twin taking its layer's row and column with the
        faces' own difference L_self - M_twin kept (peec.py:1989-2010)."""
        N = self.N
        B = sheet_blocks(self.L_self, centre[:N, :N], sums[:N, :N])
        if not len(self.twin_parent):
            return B
        lay = self.sheet_layer
        full = B[np.ix_(lay, lay)].copy()
        for m, p in enumerate(self.twin_parent):
            tw = N + m
            gap = max(self.L_self - centre[p, tw], 0.0)
            for j in range(self.n_sheets):
                if lay[j] == p and j != tw:
                    full[tw, j] = full[j, tw] = B[p, p] - gap
        return full

    def _twin_blocks(self):
        """peec.py:2012-2021."""
        N = self.N
        nx_a = self.tw_a < self.nxb
        for m, p in enumerate(self.twin_parent):
            mine = self.sheet_of_strip(self.tw_b) == N + m
            for orient, sel in (("x", nx_a), ("y", ~nx_a)):
                pick = mine & sel
                if pick.any():
                    self.blocks.append((np.column_stack([self.tw_a[pick], self.tw_b[pick]]), [int(p), N + m], orient))

    def _block_layout(self):
        """peec.py:2032-2052."""
        S = self.n_sheets
        for idx, mask, off, orient in ((self.xa, self.xb, 0, "x"), (self.ya, self.yb, self.nxb, "y")):
            if len(idx) == 0:
                continue
            sidx = -np.ones(mask.shape, np.int64)
            sidx[tuple(idx.T)] = off + np.arange(len(idx))
            bits = np.zeros(mask.shape[1:], np.int64)
            for k in range(S):
                bits |= mask[k].astype(np.int64) << k
            pos = np.nonzero(bits)
            codes = bits[pos]
            for code in np.unique(codes):
                layers = [k for k in range(S) if code >> k & 1]
                if len(layers) < 2:
                    continue
                sel = codes == code
                strips = np.stack([sidx[k, pos[0][sel], pos[1][sel]] for k in layers], axis=1)
                self.blocks.append((strips, layers, orient))

    def full_kernel(self, orient: str, t: int, s: int) -> np.ndarray:
        """Unfolded (P0, P1) spectrum from the stored quadrant (peec.py:2083-2090)."""
        Kq, P = (self.Kq["x"], self.Px) if orient == "x" else (self.Kq["y"], self.Py)
        i, j = np.arange(P[0]), np.arange(P[1])
        return Kq[np.minimum(i, P[0] - i)[:, None], np.minimum(j, P[1] - j)[None, :], t, s]

    def _full(self, orient: str, t: int, s: int) -> np.ndarray:
        cache = self.__dict__.setdefault("_full_cache", {})
        key = (orient, t, s)
        if key not in cache:
            cache[key] = self.full_kernel(orient, t, s)
        return cache[key]

    # -- L_p product (peec.py:2054-2135; FFTs on all host cores as fft_workers() = -1, peec.py:136-138)
    def Lp_matvec(self, I_s: np.ndarray) -> np.ndarray:
        out = np.empty(self.ns, complex)
        S = self.n_sheets
        for orient, idx, lo, hi, shape, P in (("x", self.xa, 0, self.nxb, (S, self.nx - 1, self.ny), self.Px),
                                              ("y", self.ya, self.nxb, self.ns, (S, self.nx, self.ny - 1), self.Py)):
            if hi <= lo:
                continue
            X = np.zeros(shape, complex)
            X[tuple(idx.T)] = I_s[lo:hi]
            F = fft2(X, s=P, axes=(1, 2), workers=FFT_WORKERS)
            G = np.zeros_like(F)
            for t in range(S):
                for s in range(S):
                    G[t] += self._full(orient, t, s) * F[s]
            Y = ifft2(G, axes=(1, 2), workers=FFT_WORKERS, overwrite_x=True)
            out[lo:hi] = Y[tuple(idx.T)]
        if self.dL is not None:             # strips narrower than the pitch (peec.py:2129-2132)
            out += self.dL * I_s
            if self.M_near is not None:
                out += self.M_near @ I_s
        return out

    # -- operators (peec.py:2150-2178, 2345-2511)
    def impedances(self, f: float):
        w = 2 * math.pi * f
        zs = np.array([complex(slab_impedance(l.thickness, f, self.sigma)) for l in self.layers])
        lay = self.sheet_layer
        R_strip = (np.concatenate([zs[lay[self.xa[:, 0]]], zs[lay[self.ya[:, 0]]]]) / self.r_width if self.ns
                   else np.zeros(0, complex))
        if len(self.tw_b):           # a split layer's face strips: the face pair's own impedance (peec.py:2161-2166)
            z_self = np.asarray(face_sheet_impedance(self.layer_t, f, self.sigma)[0])
            for tw in (self.tw_a, self.tw_b):
                R_strip[tw] = z_self[lay[self.sheet_of_strip(tw)]] / self.r_width[tw]
        if self.r_scale is not None and self.ns:       # the resistance only; the internal inductance stays
            R_strip = R_strip.real * self.r_scale + 1j * R_strip.imag
        if self.ncap:
            C, tand = self.cap[:, 4], self.cap[:, 5]
            z_cap = 1.0 / (w * C * tand + 1j * w * C) if w > 0 else np.full(self.ncap, 1e18 + 0j)
        else:
            z_cap = np.zeros(0, complex)
        z_br = np.array([b.z(f) for b in self.branches], complex)
        if self.branch_scale is not None and len(z_br):
            z_br = z_br.real * self.branch_scale + 1j * z_br.imag
        return w, R_strip, np.concatenate([z_cap, z_br])

    def set_resistance_scale(self, strips=None, branches=None):
        """Scale the strips' resistances (one factor per strip) and the branches' (their real parts), e.g. copper
        at its temperature; None: as built (peec.py:2199-2216)."""
        self.r_scale = None if strips is None else np.asarray(strips, float)
        self.branch_scale = None if branches is None else np.asarray(branches, float)
        if self.r_scale is not None and len(self.r_scale) != self.ns:
            raise ValueError(f"{len(self.r_scale)} strip factors for {self.ns} strips")
        if self.branch_scale is not None and len(self.branch_scale) != len(self.branches):
            raise ValueError(f"{len(self.branch_scale)} branch factors for {len(self.branches)} branches")
        self.r_uniform = not np.any(self.r_width != 1.0) and self.r_scale is None

    def twin_z(self, f: float) -> Optional[np.ndarray]:
        """The face coupling impedance per twin pair: z_mutual of the face pair / the strip's width
        (peec.py:2186-2197); None without split layers."""
        if not len(self.tw_b):
            return None
        z_mut = np.asarray(face_sheet_impedance(self.layer_t, f, self.sigma)[1])
        z12 = z_mut[self.sheet_layer[self.sheet_of_strip(self.tw_b)]] / self.r_width[self.tw_b]
        if self.r_scale is not None:
            z12 = z12.real * self.r_scale[self.tw_b] + 1j * z12.imag
        return z12

    def admittance(self, w, R_strip, z_tail, Z12=None) -> sp.csr_matrix:
        """peec.py:2465-2511."""
        L_own = self.L_self if self.dL is None else self.L_self + self.dL
        d = np.concatenate([1.0 / (R_strip + 1j * w * L_own), 1.0 / z_tail])
        if not self.blocks:
            return sp.diags(d).tocsr()
        z12 = None
        if Z12 is not None:
            z12 = np.zeros(self.ns, complex)
            z12[self.tw_b] = Z12
        rows, cols, vals = [np.arange(self.nb)], [np.arange(self.nb)], [d]
        in_block = np.zeros(self.nb, bool)
        for strips, layers, orient in self.blocks:
            B = (self.B_x if orient == "x" else self.B_y)[np.ix_(layers, layers)]
            m = len(layers)
            faces = [(layers.index(int(self.sheet_layer[s])), k) for k, s in enumerate(layers)
                     if s >= self.N and int(self.sheet_layer[s]) in layers] if z12 is not None else []
            if self.dL is None and self.r_uniform:       # every position alike: one inverse
                R = np.diag([R_strip[strips[0, k]] for k in range(m)]).astype(complex)
                for ia, ib in faces:
                    R[ia, ib] = R[ib, ia] = z12[strips[0, ib]]
                Zi = np.linalg.inv(R + 1j * w * B)
                Zi = np.broadcast_to(Zi.ravel(), (len(strips), m * m)).ravel()
            else:                                           # each position its own R and self inductance
                Z = np.broadcast_to(1j * w * B, (len(strips), m, m)).copy()
                Z[:, np.arange(m), np.arange(m)] += R_strip[strips] + (
                    0.0 if self.dL is None else 1j * w * self.dL[strips])
                for ia, ib in faces:
                    cross = z12[strips[:, ib]]
                    if self.dL is not None:
                        cross = cross + 1j * w * self.dL[strips[:, ib]]
                    Z[:, ia, ib] += cross
                    Z[:, ib, ia] += cross
                Zi = np.linalg.inv(Z).ravel()
            rows.append(np.repeat(strips, m, axis=1).ravel())
            cols.append(np.tile(strips, (1, m)).ravel())
            vals.append(Zi)
            in_block[strips.ravel()] = True
        vals[0] = np.where(in_block, 0.0, d)
        return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                             shape=(self.nb, self.nb))

    def operator(self, f: float) -> dict:
        """The system data and the SuperLU-factorised Schur complement at f (own factorisation, no borrowing)."""
        f = cache_value(f)
        w, R_strip, z_tail = self.impedances(f)
        Z12 = self.twin_z(f)
        Dinv = self.admittance(w, R_strip, z_tail, Z12)
        if self._base is not None:
            # a derived stack: S = S_base + U diag(1/z_new) U^T, solved by the Woodbury identity on the base's
            # factorisation (peec.py:2354-2377); only a k x k matrix is inverted
            bop = self._base.operator(f)
            k0 = self._base.nb
            U = self.ArT[:, k0:].toarray()
            SiU = bop["solve_S"](U.astype(complex))
            small_inv = np.linalg.inv(np.diag(z_tail[k0 - self.ns:]) + U.T @ SiU)

            def solve_S(v, b=bop["solve_S"], SiU=SiU, Ut=U.T, small_inv=small_inv):
                y = b(v)
                return y - SiU @ (small_inv @ (Ut @ y))
            return {"f": f, "w": w, "R_strip": R_strip, "z_tail": z_tail, "Dinv": Dinv, "S": None,
                    "solve_S": solve_S, "Z12": Z12}
        S = (self.ArT @ Dinv @ self.Ar).tocsc()
        lu = splu(S, permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=LU_PIVOT_THRESHOLD,
                  options={"SymmetricMode": True})
        return {"f": f, "w": w, "R_strip": R_strip, "z_tail": z_tail, "Dinv": Dinv, "S": S, "solve_S": lu.solve,
                "Z12": Z12}

    def matvec(self, op: dict, x: np.ndarray) -> np.ndarray:
        """[Z I - Ar V; Ar^T I] (peec.py:3043-3062)."""
        nb, ns = self.nb, self.ns
        Ib = x[:nb]
        top = np.empty(nb, complex)
        top[:ns] = op["R_strip"] * Ib[:ns] + 1j * op["w"] * self.Lp_matvec(Ib[:ns])
        if op.get("Z12") is not None:         # a split layer's faces: the slab two-port's coupling
            top[self.tw_a] += op["Z12"] * Ib[self.tw_b]
            top[self.tw_b] += op["Z12"] * Ib[self.tw_a]
        top[ns:] = op["z_tail"] * Ib[ns:]
        top -= self.Ar @ x[nb:]
        return np.concatenate([top, self.ArT @ Ib])

    def precond(self, op: dict, r: np.ndarray) -> np.ndarray:
        """Block elimination with the factorised Schur complement (peec.py:3064-3083)."""
        r1, r2 = r[: self.nb], r[self.nb:]
        y = op["solve_S"](r2 - self.ArT @ (op["Dinv"] @ r1))
        return np.concatenate([op["Dinv"] @ (r1 + self.Ar @ y), y])

    def solve(self, f: float, rhs_top: np.ndarray, J: np.ndarray, tol: float = 1e-5, max_cycles: int = 8,
              restart: Optional[int] = None, op: Optional[dict] = None):
        """(Ib, V, its, x): peec.py:2560-2607 for an unguessed solve with its own factorisation."""
        op = op if op is not None else self.operator(f)
        rhs = np.concatenate([rhs_top.astype(complex), J[self.keep].astype(complex)])
        bnorm = float(np.linalg.norm(rhs))
        if restart is None:
            restart = int(min(200, max(100, 4e8 // (16 * len(rhs)))))
        y, its, ok = gmres(lambda v: self.matvec(op, self.precond(op, v)), rhs, tol, max_cycles=max_cycles,
                           restart=restart, bnorm=bnorm, extra_cycles=GMRES_EXTRA_CYCLES)
        if not ok:
            raise OracleSolverError(f"GMRES did not converge at {f:.4g} Hz ({its} iterations)")
        x = self.precond(op, y) if y.any() else np.zeros(len(rhs), complex)
        V = np.zeros(self.n_nodes, complex)
        V[self.keep] = x[self.nb:]
        return x[: self.nb], V, its, x

    # -- coupling to the signal path (peec.py:2610-2700)
    def strip_coupling(self, trace: list) -> np.ndarray:
        d = self.d
        x, w = leggauss(3)
        q = 0.5 * x
        W = np.outer(w, w).ravel() / 4.0
        qa, ql = (g.ravel() for g in np.meshgrid(q, q, indexing="ij"))
        horiz = [s for s in trace if np.linalg.norm((s.b - s.a)[:2]) > 0]
        psi = np.zeros(self.ns)
        for axis, idx, off in ((0, self.xa, 0), (1, self.ya, self.nxb)):
            if len(idx) == 0:
                continue
            k, i, j = idx[:, 0], idx[:, 1], idx[:, 2]
            centres = np.stack([i * d + (d / 2 if axis == 0 else 0.0), j * d + (d / 2 if axis == 1 else 0.0),
                                self.sheet_z[k]], axis=1)
            acc = np.zeros(len(idx))
            half = 0.5 * self.sheet_t[k]
            for s in horiz:
                ab = s.b - s.a
                L = np.linalg.norm(ab)
                if abs(ab[axis]) < 1e-15 * L:
                    continue
                zseg = 0.5 * (s.a[2] + s.b[2])
                centres[:, 2] = self.sheet_z[k] + np.where(zseg > self.sheet_z[k], half, -half)
                rho_min = max(0.5 * s.width, 1e-7)
                a_c = segment_vector_potential(s.a, s.b, centres, rho_min)
                near = dist_to_segment(centres, s.a, s.b) < 3 * d + 2 * s.width
                if near.any():
                    c = centres[near]
                    da, dl = (qa, ql) if axis == 0 else (ql, qa)
                    pts = np.stack([c[:, 0, None] + da * d, c[:, 1, None] + dl * d,
                                    np.broadcast_to(c[:, 2, None], (len(c), len(W)))], axis=2)
                    a_q = segment_vector_potential(s.a, s.b, pts.reshape(-1, 3), rho_min).reshape(len(c), len(W))
                    a_c[near] = (a_q * W).sum(1)
                acc += (s.i * ab[axis] / L) * a_c
            psi[off: off + len(idx)] = d * acc
        return psi

    def pos(self, node) -> np.ndarray:
        k, i, j = node
        return np.array([i * self.d, j * self.d, self.zs[k]])

    def branch_coupling(self, trace: list) -> np.ndarray:
        vert = [s for s in trace if abs((s.b - s.a)[2]) > 0 and np.linalg.norm((s.b - s.a)[:2]) < 1e-12]
        out = np.zeros(self.nbr)
        for n, b in enumerate(self.branches):
            if b.kind == "via" and vert:
                pa, pb = self.pos(b.a), self.pos(b.b)
                out[n] = sum(s.i * segment_mutual(s.a, s.b, pa, pb, b.radius) for s in vert)
        return out

    def moment(self, trace: list, Ib: np.ndarray) -> np.ndarray:
        m = np.zeros(3, complex)
        for s in trace:
            m += 0.5 * s.i * np.cross(s.a, s.b)
        d = self.d
        Ix, Iy = Ib[: self.nxb], Ib[self.nxb: self.ns]
        k, _, j = self.xa.T if self.nxb else (np.zeros(0, int),) * 3
        z = self.sheet_z[k]
        m[1] += 0.5 * np.sum(z * d * Ix)
        m[2] += 0.5 * np.sum(-(j * d) * d * Ix)
        k, i, _ = self.ya.T if self.nyb else (np.zeros(0, int),) * 3
        z = self.sheet_z[k]
        m[0] += 0.5 * np.sum(-z * d * Iy)
        m[2] += 0.5 * np.sum((i * d) * d * Iy)
        I_cap = Ib[self.ns: self.ns + self.ncap]
        if len(I_cap):
            cu = self.cap[:, :4].astype(int)
            x, y = cu[:, 2] * d, cu[:, 3] * d
            dz = self.zs[cu[:, 1]] - self.zs[cu[:, 0]]
            m[0] += 0.5 * np.sum(y * dz * I_cap)
            m[1] += 0.5 * np.sum(-x * dz * I_cap)
        for b, cur in zip(self.branches, Ib[self.ns + self.ncap:]):
            m += 0.5 * np.cross(self.pos(b.a), self.pos(b.b)) * cur
        return m


def trace_self(trace: list, trace_t: float) -> float:
    """peec.py:3227-3237."""
    segs = [s for s in trace if np.linalg.norm(s.b - s.a) > 0]
    L = 0.0
    for n, si in enumerate(segs):
        L += si.i * si.i * strip_self(np.linalg.norm(si.b - si.a), si.width, trace_t)
        for sj in segs[n + 1:]:
            L += 2 * si.i * sj.i * segment_mutual(si.a, si.b, sj.a, sj.b, GMD_FLAT * (si.width + trace_t))
    return L


def trace_resistance(trace: list, f: float, sigma: float, trace_t: float) -> float:
    """peec.py:3240-3250."""
    R = 0.0
    for s in trace:
        L = np.linalg.norm(s.b - s.a)
        if L == 0 or abs(s.b[2] - s.a[2]) > 0:
            continue
        R += s.i * s.i * L / (sigma * s.width * skin_thickness(trace_t, f, sigma))
    return R


class OracleRoute:
    """peec.RouteExcitation for a driver/receiver pair (peec.py:2713-2817)."""

    def __init__(self, stack: OracleStack, trace: list, driver, receiver, trace_t: float = 35e-6):
        self.stack, self.trace, self.trace_t = stack, trace, trace_t
        ids = []
        for node, amps, what in ((driver, -1.0, "driver return node"), (receiver, 1.0, "receiver return node")):
            n = int(stack.nid[node])
            if n < 0:
                raise OracleSolverError(f"{what} is not on plane copper")
            ids.append((n, amps))
        bal: dict = {}
        for n, amps in ids:
            c = int(stack.full_label[n])
            bal[c] = bal.get(c, 0.0) + amps
        if any(abs(v) > 1e-9 for v in bal.values()):
            raise OracleSolverError("receiver return node is not connected to the driver's return node")
        self.injections = ids
        self.strip_psi = stack.strip_coupling(trace)
        self.branch_psi = stack.branch_coupling(trace)
        self.psi = np.concatenate([self.strip_psi, np.zeros(stack.ncap), self.branch_psi])
        self.L_trace = trace_self(trace, trace_t) if trace else 0.0

    def J(self) -> np.ndarray:
        J = np.zeros(self.stack.n_nodes)
        for n, amps in self.injections:
            J[n] += amps
        return J

    def rhs_top(self, f: float) -> np.ndarray:
        return -1j * 2 * math.pi * f * self.psi

    def outputs(self, f: float, Ib: np.ndarray, V: np.ndarray) -> dict:
        """Solution fields from a solved (Ib, V) (peec.py:2796-2817)."""
        st = self.stack
        w = 2 * math.pi * f
        I_x = np.zeros((st.N, st.nx - 1, st.ny), complex)
        I_y = np.zeros((st.N, st.nx, st.ny - 1), complex)
        # per layer: a split layer's two faces added (peec.py:2796-2803)
        np.add.at(I_x, tuple(st.layer_index("x").T), Ib[: st.nxb])
        np.add.at(I_y, tuple(st.layer_index("y").T), Ib[st.nxb: st.ns])
        Vg = np.zeros((st.N, st.nx, st.ny), complex)
        Vg[np.nonzero(st.node)] = V[: st.n_grid]
        v_inj = sum(amps * V[n] for n, amps in self.injections)
        Z = complex(trace_resistance(self.trace, f, st.sigma, self.trace_t) + v_inj
                    + 1j * w * (self.L_trace + np.dot(self.psi, Ib)))
        return {"I_x": I_x, "I_y": I_y, "V": Vg, "Z_loop": Z, "m": st.moment(self.trace, Ib),
                "I_branch": Ib[st.ns + st.ncap:].copy(), "I_cap": Ib[st.ns: st.ns + st.ncap].copy()}

    def solve(self, f: float, tol: float = 1e-5, restart: Optional[int] = None, op: Optional[dict] = None) -> dict:
        Ib, V, its, x = self.stack.solve(f, self.rhs_top(f), self.J(), tol=tol, restart=restart, op=op)
        out = self.outputs(f, Ib, V)
        out["its"] = its
        out["x"] = x
        return out
