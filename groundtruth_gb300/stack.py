"""The solver's Python interface, mirroring GroundTruth's (src/groundtruth/solver/peec.py):

    PlaneStack(layers, branches, capacitance, sigma, precond, screen)        peec.py:1555-1593
    PlaneStack.solve(f, rhs_top, J, tol, max_cycles, guess) -> (Ib, V, its, x)  peec.py:2513-2607
    RouteExcitation(stack, trace, inject_driver, inject_receiver, ...)       peec.py:2703-2769
    RouteExcitation.solve(f, guess) -> Solution                              peec.py:2787-2817
    PlaneProblem / MultiPlaneProblem (one-off stack + route)                 peec.py:2820-2837

with the same argument meanings, unknown numbering and error behaviour (SolverError for unsolvable models
and non-convergence, MemoryError when the device cannot hold a model).  A batched entry point,
``PlaneStack.solve_batch``, solves many (excitation, frequency) columns in one device run.

Everything per iteration runs in the CUDA library (``groundtruth_gb300/csrc``) through its C ABI
(``include/gt_gb300.h``); there is no CPU fallback: without the library the constructor raises.  The host
does the once-per-geometry index work (``layout``) and FP64 kernels (``greens``), and the cheap
per-frequency impedance tables.

Scope: the reference's current sheets (a layer with copper above and below is split into two face sheets when
``screen``); strips narrower than the pitch (the grids' wx / wy, ox / oy, rx / ry) are
modelled as the reference does (resistance over the width, dL, M_near, per-position preconditioner blocks).
"""
from __future__ import annotations

import copy
import math
import threading
from collections import OrderedDict
from dataclasses import dataclass, field
from typing import Callable, Optional

import numpy as np
import scipy.sparse as sp

from . import greens, layout

SIGMA_CU = 5.8e7
SCREEN_MIN_NODES = 16
OPERATOR_CACHE = 64           # factorised frequencies kept on the device per stack
LOWRANK_MAX = 64              # branches a derived stack may add to its base (gt_operators_derive)


class SolverError(RuntimeError):
    """A model that cannot be solved (peec.py:124-127)."""


@dataclass
class Grid:
    """One layer's copper on the shared grid (peec.py:197-223; the fields this solver reads)."""
    x0: float
    y0: float
    d: float                 # mm
    nx: int
    ny: int
    node: np.ndarray
    xb: np.ndarray
    yb: np.ndarray
    wx: Optional[np.ndarray] = None      # (nx-1, ny) copper width of each x strip, a fraction of d (None: full)
    wy: Optional[np.ndarray] = None
    ox: Optional[np.ndarray] = None      # where that copper's centre lies across the strip, a fraction of d
    oy: Optional[np.ndarray] = None
    rx: Optional[np.ndarray] = None      # the width the strip's resistance takes (None / 0: its width)
    ry: Optional[np.ndarray] = None
    fill: Optional[np.ndarray] = None    # (nx, ny) each cell's copper fraction from a sub-grid (None: whole cells)
    area: Optional[np.ndarray] = None    # (nx, ny) each node's measured copper in its cell, a fraction of d^2
    label: Optional[np.ndarray] = None   # (nx, ny) each node's net (-1: none; None: one net)
    nets: list = field(default_factory=list)   # the net names label indexes

    def xy(self, i, j):
        """Board coordinates (mm) of node (i, j), arrays too (peec.py:225-227)."""
        return self.x0 + np.asarray(i) * self.d, self.y0 + np.asarray(j) * self.d

    def nearest_node(self, x: float, y: float, max_dist: Optional[float] = None,
                     net: Optional[str] = None) -> Optional[tuple]:
        """The copper node (of `net` only, when given) nearest to (x, y) mm, None when there is none within
        max_dist (peec.py:229-255); with max_dist only a window around the point is searched."""
        mask = self.node
        if net is not None and self.label is not None:
            if net not in self.nets:
                return None
            mask = self.label == self.nets.index(net)
        ci, cj = int(round((x - self.x0) / self.d)), int(round((y - self.y0) / self.d))
        if max_dist is not None:
            r = max(int(math.ceil(max_dist / self.d)) + 1, 2)
            i0, j0 = max(ci - r, 0), max(cj - r, 0)
            ii, jj = np.nonzero(mask[i0:min(ci + r + 1, self.nx), j0:min(cj + r + 1, self.ny)])
            ii, jj = ii + i0, jj + j0
        else:
            ii, jj = np.nonzero(mask)
        if len(ii) == 0:
            return None
        px, py = self.xy(ii, jj)
        d2 = (px - x) ** 2 + (py - y) ** 2
        k = int(np.argmin(d2))
        if max_dist is not None and d2[k] > max_dist ** 2:
            return None
        return int(ii[k]), int(jj[k])

    def net_at(self, node: tuple) -> str:
        """The net of a node's copper, "" off copper or without net labels (peec.py:316-320)."""
        if self.label is None or self.label[node] < 0:
            return ""
        return self.nets[self.label[node]]

    @property
    def extent(self) -> tuple:
        """(x0, x1, y0, y1) mm that the cells cover, each node at its cell's centre (peec.py:322-327)."""
        h = self.d / 2
        return (self.x0 - h, self.x0 + (self.nx - 0.5) * self.d, self.y0 - h, self.y0 + (self.ny - 0.5) * self.d)

    def copper_area(self) -> np.ndarray:
        """Each node's copper as a share of its cell (peec.py:257-312), 0 off copper: without a measured area the
        mean width of the strips that touch it (1 at a node of full strips or of a grid without widths); with one,
        the node's run width (its x strips' mean where it has x strips on both sides and not y, and the other way
        round, else all its strips') times the measured area over the run widths summed over its 3 x 3
        neighbourhood of the same net, or the mean width where no measured copper is around it."""
        out = self.node.astype(float)
        if self.wx is None or self.wy is None:
            return out
        sx, nxs, sy, nys = (np.zeros(self.node.shape) for _ in range(4))
        sx[:-1, :] += np.where(self.xb, self.wx, 0.0)
        sx[1:, :] += np.where(self.xb, self.wx, 0.0)
        nxs[:-1, :] += self.xb
        nxs[1:, :] += self.xb
        sy[:, :-1] += np.where(self.yb, self.wy, 0.0)
        sy[:, 1:] += np.where(self.yb, self.wy, 0.0)
        nys[:, :-1] += self.yb
        nys[:, 1:] += self.yb
        n = nxs + nys
        mean_width = np.where(n > 0, (sx + sy) / np.maximum(n, 1), out)
        if self.area is None:
            return mean_width
        along_x, along_y = nxs == 2, nys == 2
        run = np.where(along_x & ~along_y, sx / np.maximum(nxs, 1),
                       np.where(along_y & ~along_x, sy / np.maximum(nys, 1), mean_width))
        a = np.where(self.node, self.area, 0.0)
        w = np.where(self.node, run, 0.0)
        net = np.where(self.node, self.label if self.label is not None else 0, -1)
        tot_a, tot_w = np.zeros(a.shape), np.zeros(a.shape)
        ni, nj = a.shape
        for di in (-1, 0, 1):
            for dj in (-1, 0, 1):
                src = (slice(max(di, 0), ni + min(di, 0)), slice(max(dj, 0), nj + min(dj, 0)))
                dst = (slice(max(-di, 0), ni + min(-di, 0)), slice(max(-dj, 0), nj + min(-dj, 0)))
                same = (net[src] == net[dst]) & (net[dst] >= 0)
                tot_a[dst] += np.where(same, a[src], 0.0)
                tot_w[dst] += np.where(same, w[src], 0.0)
        spread = np.where(tot_w > 0, w * tot_a / np.maximum(tot_w, 1e-12), 0.0)
        return np.where(self.node, np.where(spread > 0, spread, mean_width), 0.0)


@dataclass
class PlaneLayer:
    name: str
    z: float
    grid: Grid
    thickness: float = 35e-6


@dataclass
class Branch:
    a: tuple
    b: tuple
    z: Callable[[float], complex]
    name: str = ""
    kind: str = "part"
    radius: float = 1.5e-4


VIA_PLATING = 25e-6           # m, a via barrel's plating (peec.py:75)


def via_impedance(length_m: float, drill_m: float, sigma: float = SIGMA_CU, filled: bool = False,
                  plating: float = VIA_PLATING) -> Callable[[float], complex]:
    """A plated via barrel between two layers as a branch impedance z(f) = R + j w L (peec.py:1061-1072): L the
    partial self inductance of a filament at the barrel's radius (a thin tube's GMD), R the plating ring's (the
    whole hole's when a pin fills it)."""
    r = max(drill_m / 2, 5e-5)
    length = max(length_m, 1e-6)
    L = float(greens.filament_mutual(length, np.array(0.0), np.array(r)))
    area = math.pi * r * r if filled else math.pi * 2 * r * plating
    R = length / (sigma * area)
    return lambda f, R=R, L=L: complex(R, 2 * math.pi * f * L)


def track_impedance(length_m: float, width_m: float, thickness_m: float = 35e-6,
                    sigma: float = SIGMA_CU) -> Callable[[float], complex]:
    """A piece of track as a lumped branch (a bridge across another net's cells, peec.py:1075-1090): the
    resistance over the copper's effective thickness at f (skin depth) + j w its partial self inductance."""
    length = max(length_m, 1e-6)
    L = greens.strip_self(length, width_m, thickness_m)

    def z(f: float) -> complex:
        t = float(greens.skin_thickness(thickness_m, f, sigma))
        return complex(length / (sigma * width_m * t), 2 * math.pi * f * L)
    return z


@dataclass
class PlanePair:
    upper: int
    lower: int
    c_per_area: float
    tan_delta: float = 0.02


@dataclass
class TraceSegment:
    a: np.ndarray
    b: np.ndarray
    width: float
    i: float = 1.0


@dataclass
class Solution:
    """One solve at one frequency per A of loop current (peec.py:1092-1115)."""
    f: float
    I_x: np.ndarray
    I_y: np.ndarray
    V: np.ndarray
    I_branch: np.ndarray
    Z_loop: complex
    m: np.ndarray
    iterations: int
    I_cap: np.ndarray = field(default_factory=lambda: np.zeros(0, complex))
    residual: float = 0.0          # final relative FP64 residual ||b - K x|| / ||b||
    I_twin: Optional[np.ndarray] = None   # (2, pairs) a split layer's upper- and lower-face strip currents
    W_x: Optional[np.ndarray] = None      # per layer the strips' resistance widths (None: all full)
    W_y: Optional[np.ndarray] = None
    A_cu: Optional[np.ndarray] = None     # per layer each node's copper share of its cell

    @property
    def L_loop(self) -> float:
        return self.Z_loop.imag / (2 * math.pi * self.f)

    def node_field(self, k: int, d_mm: float, copper: bool = False) -> tuple:
        """Complex (Kx, Ky) at the nodes of layer k in A/m per A (peec.py:1151-1203): each node averages the
        strips of each direction that touch it and carry current, per cell width; copper=True per width of the
        copper itself, the vector's length set by the touching strips' heat over the node's copper area."""
        d = d_mm * 1e-3
        Ix, Iy = self.I_x[k], self.I_y[k]
        wx = wy = None
        if copper and self.W_x is not None:
            wx, wy = self.W_x[k], self.W_y[k]
            Ix, Iy = Ix / wx, Iy / wy
        nx, ny = self.V.shape[1:]
        kx, ky = np.zeros((nx, ny), complex), np.zeros((nx, ny), complex)
        cx, cy = np.zeros((nx, ny)), np.zeros((nx, ny))
        kx[:-1, :] += Ix
        kx[1:, :] += Ix
        cx[:-1, :] += Ix != 0
        cx[1:, :] += Ix != 0
        ky[:, :-1] += Iy
        ky[:, 1:] += Iy
        cy[:, :-1] += Iy != 0
        cy[:, 1:] += Iy != 0
        kx, ky = kx / np.maximum(cx, 1) / d, ky / np.maximum(cy, 1) / d
        if not copper or self.A_cu is None:
            return kx, ky
        # the node's share of its strips' heat per rho / t, sum 1/2 |I|^2 / width, over its copper area
        hx = 0.5 * np.abs(self.I_x[k]) ** 2 / (wx if wx is not None else 1.0)
        hy = 0.5 * np.abs(self.I_y[k]) ** 2 / (wy if wy is not None else 1.0)
        q = np.zeros((nx, ny))
        q[:-1, :] += hx
        q[1:, :] += hx
        q[:, :-1] += hy
        q[:, 1:] += hy
        a = self.A_cu[k].astype(float)
        mag = np.sqrt(np.where(a > 0, q / np.maximum(a, 1e-12), 0.0)) / d
        vec = np.sqrt(np.abs(kx) ** 2 + np.abs(ky) ** 2)
        # the mean's direction at that length; where the mean cancels, the length alone along x
        scale = np.where(vec > 1e-9 * mag, mag / np.maximum(vec, 1e-300), 0.0)
        alone = (vec <= 1e-9 * mag) & (mag > 0)
        return np.where(alone, mag, kx * scale), np.where(alone, 0.0, ky * scale)

    def state_for(self, stack: "PlaneStack") -> np.ndarray:
        """The solver's unknown vector [branch currents; kept node potentials] of this solution on `stack`, the
        stack it was solved on, rebuilt from the currents and potentials kept here (peec.py:1127-1145; a warm
        start for a derived stack through map_state)."""
        strips = np.concatenate([self.I_x[tuple(stack.layer_index("x").T)], self.I_y[tuple(stack.layer_index("y").T)]])
        if len(stack.tw_b):
            # a split layer's faces: I_x / I_y hold their sum (peec.py:1135-1140)
            if self.I_twin is not None and self.I_twin.shape[1] == len(stack.tw_b):
                strips[stack.tw_a], strips[stack.tw_b] = self.I_twin
            else:
                strips[stack.tw_b] = 0.0
        Ib = np.concatenate([strips, self.I_cap, self.I_branch])
        return np.concatenate([Ib, self.V[np.nonzero(stack.node)][stack.keep]])

    def sheet_current(self, k: int, d_mm: float, copper: bool = False) -> np.ndarray:
        """|K| at the nodes of layer k (peec.py:1205-1208)."""
        kx, ky = self.node_field(k, d_mm, copper)
        return np.sqrt(np.abs(kx) ** 2 + np.abs(ky) ** 2)

    def dominant_phase(self) -> float:
        """The phase at which the plane currents are largest (peec.py:1210-1226): half the angle of the sum of
        the strip currents squared over all layers (the principal axis of the currents in the complex plane),
        turned by pi where the currents at that phase run against the signal's own (their real part); 0 for
        currents that are all zero."""
        phi = getattr(self, "_phase", None)
        if phi is not None:
            return phi
        sq = complex(np.sum(self.I_x ** 2) + np.sum(self.I_y ** 2))
        phi = 0.5 * math.atan2(sq.imag, sq.real) if abs(sq) > 0 else 0.0
        turn = np.exp(-1j * phi)
        if float(np.sum((self.I_x * turn).real * self.I_x.real) + np.sum((self.I_y * turn).real * self.I_y.real)) < 0:
            phi += math.pi
        self._phase = phi
        return phi

    def sheet_vectors(self, k: int, d_mm: float, copper: bool = False) -> tuple:
        """Real (Kx, Ky) at the nodes of layer k at the dominant phase (peec.py:1228-1233)."""
        kx, ky = self.node_field(k, d_mm, copper)
        turn = np.exp(-1j * self.dominant_phase())
        return (kx * turn).real, (ky * turn).real

    def layer_share(self, masks: Optional[list] = None) -> np.ndarray:
        """Each layer's share of the summed strip current magnitudes; masks: per layer (x, y) strip masks to count
        (peec.py:1235-1247)."""
        per = np.zeros(len(self.I_x))
        for k in range(len(self.I_x)):
            ax, ay = np.abs(self.I_x[k]), np.abs(self.I_y[k])
            if masks is not None:
                ax, ay = ax * masks[k][0], ay * masks[k][1]
            per[k] = ax.sum() + ay.sum()
        total = per.sum()
        return per / total if total > 0 else per


def native_geometry(st):
    from . import native
    return native.Geometry(st)


PRECOND_REUSE = 0.25      # peec.py: the log-frequency window a factorisation may serve


def borrow_plan(keys: list) -> list:
    """For each frequency, the index of the frequency whose factorisation preconditions it: along the sorted
    sweep every other frequency borrows the factorisation next below it when that one is within PRECOND_REUSE
    (|ln f / f_lu|) and lends to no one else yet (peec.py:2227-2343 decides borrowing between rounds; within one
    batch this halves the factorisations of a sweep whose frequencies are close)."""
    order = sorted(range(len(keys)), key=lambda q: keys[q])
    plan = list(range(len(keys)))
    last_own, lent = None, False
    for q in order:
        if last_own is not None and not lent and keys[last_own] > 0 and keys[q] > 0 \
                and abs(math.log(keys[q] / keys[last_own])) < PRECOND_REUSE:
            plan[q] = last_own
            lent = True
        else:
            last_own, lent = q, False
    return plan


def freq_key(f: float) -> float:
    """f to 12 significant digits (peec.py:2292-2296, 3264-3267)."""
    return float(f"{float(f):.12g}")


class PlaneStack:
    """Plane layers with their branches and plane-pair capacitance on one GPU."""

    def __init__(self, layers: list, branches: Optional[list] = None, capacitance: Optional[list] = None,
                 sigma: float = SIGMA_CU, precond: str = "diag", screen: bool = True, *, leaf: int = 48,
                 _device: bool = True):
        from . import native
        if not layers:
            raise SolverError("no plane layers")
        if precond not in ("diag", "sheet"):
            raise ValueError("precond must be 'diag' or 'sheet'")
        g0 = layers[0].grid
        for l in layers:
            if (l.grid.nx, l.grid.ny, l.grid.d) != (g0.nx, g0.ny, g0.d):
                raise SolverError("all layers must share one grid")
        self.lib = native.load() if _device else None
        self._device = bool(_device)
        self.screen, self.leaf = screen, leaf
        self._base: Optional[PlaneStack] = None
        self.n_lowrank = 0
        self.layers = list(layers)
        self.N = len(layers)
        self.nx, self.ny = g0.nx, g0.ny
        self.d = g0.d * 1e-3
        self.zs = np.array([l.z for l in layers], float)
        self.ts = np.array([l.thickness for l in layers], float)
        self.sigma = sigma
        self.precond_mode = precond
        self.pairs = list(capacitance or [])
        self._faces(np.stack([l.grid.node for l in layers]).astype(bool), screen)
        self.branches_all = list(branches or [])
        t, kept = layout.topology([l.grid.node for l in layers], [l.grid.xb for l in layers],
                                  [l.grid.yb for l in layers], self.d,
                                  [(p.upper, p.lower, p.c_per_area, p.tan_delta) for p in self.pairs],
                                  [(b.a, b.b) for b in self.branches_all], self.twin_parent,
                                  [l.grid.fill for l in layers])
        self.top = t
        self.branches = [self.branches_all[k] for k in kept]
        self.node, self.nid, self.xa, self.ya, self.keep = t.node, t.nid, t.xa, t.ya, t.keep
        self.nxb, self.nyb, self.ns, self.ncap, self.nbr, self.nb = t.nxb, len(t.ya), t.ns, t.ncap, t.nbr, t.nb
        self.n_nodes = self.n_grid = t.n_nodes
        self.full_label, self.cond_label = t.full_label, t.cond_label
        self._twins()
        self.dense = layout.dense_layout(t)
        self._kernels()
        self.r_scale = self.branch_scale = None
        self._widths()
        self._corrections()
        # per layer the strips' resistance widths and the nodes' copper shares (Solution.node_field(copper=True))
        self.A_cu = np.stack([l.grid.copper_area() for l in self.layers]).astype(np.float32)
        self.W_x = self.W_y = None
        if np.any(self.strip_width != 1.0) or np.any(self.r_width != 1.0):
            self.W_x, self.W_y = np.ones((self.N, self.nx - 1, self.ny)), np.ones((self.N, self.nx, self.ny - 1))
            self.W_x[tuple(self.layer_index("x").T)] = self.r_width[: self.nxb]
            self.W_y[tuple(self.layer_index("y").T)] = self.r_width[self.nxb:]
        self._schur_structure(leaf)
        self._lock = threading.Lock()
        self._ops: OrderedDict = OrderedDict()
        # keep only the FP32 copies of the factor panels (a third of the memory): for stacks that only take
        # "mixed" solves and are not the base of derived stacks (native.Operators(fp32_panels=True))
        self.fp32_panels = False
        self.handle = native_geometry(self) if _device else None

    # ------------------------------------------------------------------ construction
    def _faces(self, node: np.ndarray, screen: bool):
        """The current sheets (peec.py:1658-1697): one per layer, and a second for each layer with copper of other
        layers above and below at SCREEN_MIN_NODES or more of its nodes (when `screen`): such a layer is split into
        its two faces, its own sheet at the upper face and the twin (numbered after the layers) at the lower one,
        both with all its strips on its nodes.  Sets twin_parent, n_sheets, sheet_layer, sheet_z (the height each
        sheet's current stands at) and sheet_t (the copper face_gap takes off: 0 for a face sheet)."""
        N = self.N
        twins = []
        if screen and N >= 3:
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
        z, st = self.zs.copy(), self.ts.copy()
        z[twins] = self.zs[twins] + 0.5 * self.ts[twins]
        st[twins] = 0.0
        self.sheet_z = np.concatenate([z, self.zs[twins] - 0.5 * self.ts[twins]])
        self.sheet_t = np.concatenate([st, np.zeros(len(twins))])

    def _twins(self):
        """tw_a / tw_b: the strips of each split layer's upper face and of its twin, pairwise (peec.py:1699-1716),
        and each strip's twin-pair index (tw_of, -1 for a one-sheet layer's strip)."""
        N, t = self.N, self.top
        a, b = [], []
        for xb, lo in ((t.xb, 0), (t.yb, self.nxb)):
            per = np.count_nonzero(xb.reshape(self.n_sheets, -1), axis=1)
            start = lo + np.concatenate([[0], np.cumsum(per)[:-1]])
            for m, p in enumerate(self.twin_parent):
                a.append(start[p] + np.arange(per[p]))
                b.append(start[N + m] + np.arange(per[p]))
        self.tw_a = np.concatenate(a).astype(np.int64) if a else np.zeros(0, np.int64)
        self.tw_b = np.concatenate(b).astype(np.int64) if b else np.zeros(0, np.int64)

    def sheet_of_strip(self, strips: np.ndarray) -> np.ndarray:
        strips = np.asarray(strips, np.int64)
        out = np.empty(len(strips), np.int64)
        x = strips < self.nxb
        out[x] = self.xa[strips[x], 0]
        out[~x] = self.ya[strips[~x] - self.nxb, 0]
        return out

    def layer_index(self, orient: str) -> np.ndarray:
        """The orientation's strips as (layer, i, j) rows (peec.py:1718-1729)."""
        idx = (self.xa if orient == "x" else self.ya).copy()
        idx[:, 0] = self.sheet_layer[idx[:, 0]]
        return idx

    def face_z(self, k: int, z: float) -> float:
        """Sheet k's face towards height z (m): a one-sheet layer's centre moved half its copper towards z, a face
        sheet's own height (its sheet_t is 0) (peec.py:1935-1939)."""
        t = 0.5 * self.sheet_t[k]
        return self.sheet_z[k] + (t if z > self.sheet_z[k] else -t)

    def surface_impedance(self, f: float, t: float) -> complex:
        """Sheet impedance (ohm per square) of copper t thick at f: the one-face slab (peec.py:2144-2148)."""
        return complex(greens.slab_impedance(t, f, self.sigma))

    def face_gap(self, s: int, t: int) -> float:
        """The distance between the faces sheets s and t turn to each other (peec.py:1926-1933)."""
        if s == t:
            return 0.0
        return max(abs(self.sheet_z[s] - self.sheet_z[t]) - 0.5 * (self.sheet_t[s] + self.sheet_t[t]), 1e-6)

    def _kernels(self):
        """Strip kernels per sheet pair and their spectra at this build's FFT sizes (peec.py:1941-1988)."""
        nx, ny, S = self.nx, self.ny, self.n_sheets
        d = greens.round12(self.d)
        self.P = {"x": (greens.fft_size(2 * (nx - 1) - 1), greens.fft_size(2 * ny - 1)),
                  "y": (greens.fft_size(2 * nx - 1), greens.fft_size(2 * (ny - 1) - 1))}
        spec = {o: np.zeros((self.P[o][1] // 2 + 1, self.P[o][0] // 2 + 1, S, S)) for o in "xy"}
        centre, sx, sy = np.zeros((S, S)), np.zeros((S, S)), np.zeros((S, S))
        cache: dict = {}
        for s in range(S):
            for t in range(s, S):
                dz = greens.round12(self.face_gap(s, t))
                if dz not in cache and self._device:
                    # on the device (gt_kernel_spectrum): the centre is the nearest tape value, the sums the
                    # spectra's DC terms
                    from . import native
                    nxv, nyv = greens.near_values(nx - 1, ny, d, dz), greens.near_values(ny - 1, nx, d, dz)
                    px, py = self.P["x"], self.P["y"]
                    qxq = native.kernel_spectrum(nx - 1, ny, d, dz, px[0], px[1], nxv)
                    qyq = native.kernel_spectrum(ny - 1, nx, d, dz, py[1], py[0], nyv).T
                    cache[dz] = (qxq.T, qyq.T, float(nxv[0, 0]), float(qxq[0, 0]), float(qyq[0, 0]))
                elif dz not in cache:
                    kx = greens.strip_kernel(nx - 1, ny, d, dz)
                    ky = greens.strip_kernel(ny - 1, nx, d, dz).T
                    cache[dz] = (greens.spectrum_quadrant(kx, *self.P["x"]).T, greens.spectrum_quadrant(ky, *self.P["y"]).T,
                                 float(kx[nx - 2, ny - 1]), float(kx.sum()), float(ky.sum()))
                qx, qy, c, a, b = cache[dz]
                spec["x"][:, :, s, t] = spec["x"][:, :, t, s] = qx
                spec["y"][:, :, s, t] = spec["y"][:, :, t, s] = qy
                centre[s, t] = centre[t, s] = c
                sx[s, t] = sx[t, s] = a
                sy[s, t] = sy[t, s] = b
        dz0 = greens.round12(0.0)
        self.L_self = cache[dz0][2] if dz0 in cache else float(greens.strip_kernel(nx - 1, ny, d, 0.0)[nx - 2, ny - 1])
        # layout (Q1, Q0, S, S): the column pass reads one pixel column's quadrant rows contiguously; scaled by
        # the inverse transform's 1 / (P0 P1)
        self.spectrum = {o: np.ascontiguousarray(spec[o] / (self.P[o][0] * self.P[o][1])) for o in "xy"}
        self.centre, self.sum_x, self.sum_y = centre, sx, sy
        self.B = None
        self.twin_diag = False
        if self.precond_mode == "sheet" and self.N > 1:
            self.B = {"x": self._sheet_block(centre, sx), "y": self._sheet_block(centre, sy)}
        elif len(self.twin_parent):
            # 'diag' with split layers: each face pair at a position is a 2 x 2 block with their own and mutual
            # partial inductance (peec.py:1979-1987)
            B = np.diag(np.full(S, self.L_self))
            for m, p in enumerate(self.twin_parent):
                B[p, self.N + m] = B[self.N + m, p] = centre[p, self.N + m]
            self.B = {"x": B, "y": B}
            self.twin_diag = True

    def _sheet_block(self, centre: np.ndarray, sums: np.ndarray) -> np.ndarray:
        """The 'sheet' block over every sheet: made over the layers, a split layer's twin taking its layer's row
        and column, the two faces keeping their own difference L_self - M_twin (peec.py:1989-2010)."""
        N = self.N
        B = greens.sheet_blocks(self.L_self, centre[:N, :N], sums[:N, :N])
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

    def _dinv_block(self, name: str, lay: list, R: np.ndarray, dl: np.ndarray, z12: dict, w: float) -> np.ndarray:
        """D^-1 of the strips at one position (peec.py:2465-2511): present sheets `lay`, their impedances R and
        self-inductance changes dl, the face couplings z12 {twin sheet: coupling} -> the S x S block.  A 'sheet'
        block over all present sheets, a 2 x 2 block per face pair ('diag' with split layers), else diagonal."""
        S, N = self.n_sheets, self.N
        blk = np.zeros((S, S), complex)
        if self.B is not None and not self.twin_diag and len(lay) >= 2:
            groups = [list(range(len(lay)))]
        elif self.twin_diag:
            groups, used = [], set()
            for q, k in enumerate(lay):
                if k >= N and int(self.sheet_layer[k]) in lay:
                    qa = lay.index(int(self.sheet_layer[k]))
                    groups.append([qa, q])
                    used |= {qa, q}
            groups += [[q] for q in range(len(lay)) if q not in used]
        else:
            groups = [[q] for q in range(len(lay))]
        for g in groups:
            sh = [lay[q] for q in g]
            if len(g) == 1:
                blk[sh[0], sh[0]] = 1.0 / (R[g[0]] + 1j * w * (self.L_self + dl[g[0]]))
                continue
            Z = 1j * w * self.B[name][np.ix_(sh, sh)] + np.diag(R[g] + 1j * w * dl[g])
            for ib, k in enumerate(sh):
                if k >= N and int(self.sheet_layer[k]) in sh:
                    ia = sh.index(int(self.sheet_layer[k]))
                    cross = z12[k] + 1j * w * dl[g[ib]] * (self.dL is not None)
                    Z[ia, ib] += cross
                    Z[ib, ia] += cross
            blk[np.ix_(sh, sh)] = np.linalg.inv(Z)
        return blk

    def _widths(self):
        """Strips narrower than the pitch (peec.py:1732-1843): strip_width and r_width per strip (fractions of
        the pitch), dL (the self-inductance change, None when every strip is full) and M_near (sparse side-by-side
        mutual changes, with a split layer's faces sharing them).  _corrections makes the device's view."""
        t, S = self.top, self.n_sheets
        sx, sy = (self.nx - 1, self.ny), (self.nx, self.ny - 1)
        lx, ly = self.layer_index("x"), self.layer_index("y")      # a face sheet has its layer's copper

        def gather(attr, idx, shape, default):
            if len(idx) == 0:
                return np.zeros(0)
            if all(getattr(l.grid, attr, None) is None for l in self.layers):
                return np.full(len(idx), default)
            w = np.stack([np.asarray(getattr(l.grid, attr), float) if getattr(l.grid, attr, None) is not None
                          else np.full(shape, default) for l in self.layers])
            return w[tuple(idx.T)]
        w = np.concatenate([gather("wx", lx, sx, 1.0), gather("wy", ly, sy, 1.0)])
        ok = w > 0
        self.strip_width = np.where(ok, w, 1.0)
        rw = np.concatenate([gather("rx", lx, sx, 0.0), gather("ry", ly, sy, 0.0)])
        self.r_width = np.where(ok & (rw > 0), rw, self.strip_width)
        off = np.where(ok, np.concatenate([gather("ox", lx, sx, 0.0), gather("oy", ly, sy, 0.0)]), 0.0)
        self.dL = self.M_near = None
        narrow = self.strip_width < 1.0
        if np.any(narrow):
            th = self.ts[np.concatenate([lx[:, 0], ly[:, 0]])]
            dL = np.zeros(self.ns)
            keys, inv = np.unique(np.round(np.column_stack([self.strip_width[narrow], th[narrow]]), 12), axis=0,
                                  return_inverse=True)
            dL[narrow] = greens.narrow_self(self.d, keys[:, 0], keys[:, 1])[np.ravel(inv)]
            self.dL = dL
            rows, cols, steps = [], [], []
            for idx, shape, lo, axis in ((t.xa, sx, 0, 2), (t.ya, sy, self.nxb, 1)):
                if len(idx) == 0:
                    continue
                at = -np.ones((S, *shape), np.int64)
                at[tuple(idx.T)] = lo + np.arange(len(idx))
                n_ax = shape[0] if axis == 2 else shape[1]
                for k in range(-greens.NEAR_AXIAL, greens.NEAR_AXIAL + 1):
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
            if len(a):
                k = np.concatenate(steps)
                wa, wb = self.strip_width[a], self.strip_width[b]
                gap = 1.0 + off[b] - off[a]
                keys, inv = np.unique(np.round(np.column_stack([wa, wb, gap, k]), 9), axis=0, return_inverse=True)
                one = np.ones(len(keys))
                dM = (greens.side_mutual(self.d, keys[:, 0], keys[:, 1], keys[:, 2], keys[:, 3])
                      - greens.side_mutual(self.d, one, one, one, keys[:, 3]))[np.ravel(inv)]
                M = sp.coo_matrix((dM, (a, b)), shape=(self.ns, self.ns))
                self.M_near = (M + M.T).tocsr()
            if len(self.tw_b):
                # a split layer's faces share their copper's corrections (peec.py:1822-1843)
                n = self.ns
                pairs = np.concatenate([self.tw_a, self.tw_b]), np.concatenate([self.tw_b, self.tw_a])
                extra = sp.coo_matrix((np.concatenate([self.dL[self.tw_a], self.dL[self.tw_b]]), pairs),
                                      shape=(n, n))
                if self.M_near is not None:
                    swap = sp.coo_matrix((np.ones(len(pairs[0])), pairs), shape=(n, n)).tocsr()
                    extra = extra + self.M_near @ swap
                self.M_near = ((self.M_near if self.M_near is not None else 0) + extra).tocsr()

    def _corrections(self):
        """The device's view of the strips that are not full squares (narrow, a resistance width or factor):
        the positions whose D^-1 blocks are their own (override) and the rows of the system product's corrections
        (with a split layer's face partners)."""
        t = self.top
        sx, sy = (self.nx - 1, self.ny), (self.nx, self.ny - 1)
        sc = self.r_scale if self.r_scale is not None else np.ones(self.ns)
        odd = (self.strip_width != 1.0) | (self.r_width != 1.0) | (sc != 1.0)
        if self.dL is not None:
            odd |= self.dL != 0
        self.override = {"x": -np.ones(sx, np.int32), "y": -np.ones(sy, np.int32)}
        self.override_pos = []            # (orientation 0 / 1, i, j) per override block
        for o, (name, idx, lo) in enumerate((("x", t.xa, 0), ("y", t.ya, self.nxb))):
            if len(idx) == 0:
                continue
            sel = odd[lo: lo + len(idx)]
            pos = np.unique(idx[sel][:, 1:], axis=0)
            for i, j in pos:
                self.override[name][i, j] = len(self.override_pos)
                self.override_pos.append((o, int(i), int(j)))
        self.n_override = len(self.override_pos)
        # correction rows: strips with a resistance factor, a self change, side-by-side changes or a face partner
        partner = -np.ones(self.ns, np.int64)
        partner[self.tw_a], partner[self.tw_b] = self.tw_b, self.tw_a
        twin = -np.ones(self.ns, np.int64)
        tw_fac = np.zeros(self.ns)
        pair_sc = np.ones(self.ns)        # a face pair's coupling takes its lower strip's factor (peec.py:2196)
        if len(self.tw_b):
            m = self.sheet_of_strip(self.tw_b) - self.N
            twin[self.tw_a], twin[self.tw_b] = m, m
            tw_fac[self.tw_a] = tw_fac[self.tw_b] = 1.0 / self.r_width[self.tw_b]
            pair_sc[self.tw_a] = pair_sc[self.tw_b] = sc[self.tw_b]
        rows = np.flatnonzero(odd | (partner >= 0) | (np.diff(self.M_near.indptr) > 0 if self.M_near is not None
                                                       else np.zeros(self.ns, bool)))
        c2d = self.dense.compact_to_dense
        M = self.M_near[rows] if self.M_near is not None else sp.csr_matrix((len(rows), max(self.ns, 1)))
        self.narrow_rows = {
            "pos": c2d[rows].astype(np.int64),
            "sheet": np.concatenate([t.xa[:, 0], t.ya[:, 0]])[rows].astype(np.int32) if len(rows) else np.zeros(0, np.int32),
            "rdelta": 1.0 / self.r_width[rows] - 1.0,
            "dl": self.dL[rows] if self.dL is not None else np.zeros(len(rows)),
            "ptr": M.indptr.astype(np.int64),
            "col": c2d[M.indices].astype(np.int64),
            "val": M.data.astype(np.float64),
            "partner": np.where(partner[rows] >= 0, c2d[np.maximum(partner[rows], 0)], -1).astype(np.int64),
            "twin": np.maximum(twin[rows], 0).astype(np.int32),
            "tw_fac": tw_fac[rows],
            # a resistance factor scales the real part only: R = (Re z sc + j Im z) / w
            "rre": (sc[rows] - 1.0) / self.r_width[rows],
            "twre": (pair_sc[rows] - 1.0) * tw_fac[rows],
        }

    def _schur_structure(self, leaf: int, sym=None):
        """S = Ar^T D^-1 Ar as a linear map of the per-frequency admittance table, and its symbolic analysis."""
        t, S, nx, ny = self.top, self.n_sheets, self.nx, self.ny
        nxy = nx * ny
        self.sheet = self.B is not None
        lay = self.sheet_layer
        ncode = 1 << S
        self.code = {"x": np.zeros((nx - 1, ny), np.uint8), "y": np.zeros((nx, ny - 1), np.uint8)}
        for k in range(S):
            self.code["x"] |= (t.xb[k].astype(np.uint8) << k)
            self.code["y"] |= (t.yb[k].astype(np.uint8) << k)
        self.tab_ovr0 = 2 * ncode * S * S
        self.tab_cap0 = self.tab_ovr0 + self.n_override * S * S
        self.tab_br0 = self.tab_cap0 + len(t.pair_layers)
        self.n_table = self.tab_br0 + self.nbr
        kept_of_nid = -np.ones(t.n_nodes, np.int64)
        kept_of_nid[t.keep] = np.arange(t.n_keep)
        U, Vv, T, C = [], [], [], []

        def add(s1_nodes, s2_nodes, tab, scale=None):
            """D^-1 entry tab (times scale) between strips with ends s1 (a, b) and s2 (a, b): all (u, v) terms."""
            for (u, su) in ((s1_nodes[0], 1.0), (s1_nodes[1], -1.0)):
                for (v, sv) in ((s2_nodes[0], 1.0), (s2_nodes[1], -1.0)):
                    ku, kv = kept_of_nid[u], kept_of_nid[v]
                    ok = (ku >= 0) & (kv >= 0)
                    U.append(ku[ok]); Vv.append(kv[ok]); T.append(tab[ok])
                    C.append(su * sv * scale[ok] if scale is not None else np.full(int(ok.sum()), su * sv))

        for o, idx, di, dj in ((0, t.xa, 1, 0), (1, t.ya, 0, 1)):
            if len(idx) == 0:
                continue
            k, i, j = idx[:, 0], idx[:, 1], idx[:, 2]
            code = self.code["x" if o == 0 else "y"][i, j].astype(np.int64)
            ends1 = (t.nid[lay[k], i, j], t.nid[lay[k], i + di, j + dj])     # a strip joins its layer's nodes
            partners = range(S) if self.sheet else [None]
            for l in partners:
                if l is None:                      # diagonal D: each strip with itself
                    ll = k
                    sel = np.ones(len(k), bool)
                else:                              # blocks: every strip present at the same position (with split
                    ll = np.full(len(k), l)        # layers under 'diag': only a face pair)
                    sel = (code >> l) & 1 == 1
                    if self.twin_diag:
                        sel &= lay[k] == lay[l]
                ovr = self.override["x" if o == 0 else "y"][i, j].astype(np.int64)
                tab = np.where(ovr >= 0, self.tab_ovr0 + (ovr * S + k) * S + ll, ((o * ncode + code) * S + k) * S + ll)
                e1 = (ends1[0][sel], ends1[1][sel])
                e2 = (t.nid[lay[ll[sel]], i[sel], j[sel]], t.nid[lay[ll[sel]], i[sel] + di, j[sel] + dj])
                add(e1, e2, tab[sel])
        cu = t.cap[:, :4].astype(np.int64)
        if len(cu):
            pidx = np.concatenate([np.full(int(t.cap_mask[p].sum()), p) for p in range(len(t.pair_layers))])
            e = (t.nid[cu[:, 0], cu[:, 2], cu[:, 3]], t.nid[cu[:, 1], cu[:, 2], cu[:, 3]])
            # a partly covered cell's admittance: the pair's whole-cell one times the facing share
            add(e, e, self.tab_cap0 + pidx, t.cap_share if np.any(t.cap_share != 1.0) else None)
        if self.nbr:
            e = (t.branch_ab[:, 0], t.branch_ab[:, 1])
            add(e, e, self.tab_br0 + np.arange(self.nbr))
        U, Vv, T, C = (np.concatenate(a) for a in (U, Vv, T, C))
        n = t.n_keep
        pattern = sp.coo_matrix((np.ones(len(U)), (U, Vv)), shape=(n, n)).tocsr()
        pattern = ((pattern + pattern.T) != 0).astype(np.float64)
        self.sym = sym if sym is not None else layout.symbolic(t, pattern, leaf)
        sym = self.sym
        # kept index -> factor index
        node_dense = np.flatnonzero(t.node.ravel())
        fac = sym.perm[node_dense[t.keep]]
        fu, fv = fac[U], fac[Vv]
        low = fu >= fv
        fu, fv, T, C = fu[low], fv[low], T[low], C[low]
        # S entry index of (row, col) in the symbolic's column-major lower list
        key_s = sym.s_col * n + sym.s_row
        e = np.searchsorted(key_s, fv * n + fu)
        assert np.all(key_s[e] == fv * n + fu)
        M = sp.coo_matrix((C, (e, T)), shape=(len(key_s), self.n_table)).tocsr()
        M.sum_duplicates()
        M.eliminate_zeros()
        self.sterm = M

    # ------------------------------------------------------------------ derived stacks
    def node_id(self, node) -> int:
        """The node number of (layer, i, j), -1 when it is not on copper (peec.py:1864-1869)."""
        k, i, j = (int(v) for v in node)
        if not (0 <= k < self.N and 0 <= i < self.nx and 0 <= j < self.ny):
            return -1
        return int(self.nid[k, i, j])

    def with_branches(self, extra: list, device: Optional[bool] = None) -> "PlaneStack":
        """This stack plus a few branches (candidate vias, parts), peec.py:1871-1912.  Shares the grids, the
        kernel spectra and the Schur structure; its solves reuse this stack's factorisations through a low-rank
        (Woodbury) update of the Schur complement (gt_operators_derive).  Branches with an end off copper or
        both ends on one node are dropped; none left: this stack.  A branch that joins two pieces of copper
        changes the reference nodes: a stack of its own.  A derived stack of a derived stack derives from the
        first base with all the added branches (the same system and preconditioner).  device=False: the host
        side only (numbering, couplings, outputs), without a device geometry."""
        extra = [b for b in extra if self.node_id(b.a) >= 0 and self.node_id(b.b) >= 0
                 and tuple(b.a) != tuple(b.b)]
        if not extra:
            return self
        a = np.array([self.node_id(b.a) for b in extra])
        b = np.array([self.node_id(b.b) for b in extra])
        branches = self.branches + extra
        root = self._base if self._base is not None else self
        if np.any(self.full_label[a] != self.full_label[b]) or len(branches) - root.nbr > LOWRANK_MAX:
            return PlaneStack(self.layers, branches, self.pairs, self.sigma, self.precond_mode, self.screen,
                              leaf=self.leaf, _device=self._device if device is None else bool(device))
        t = layout.add_branches(root.top, [(self.node_id(br.a), self.node_id(br.b)) for br in branches[root.nbr:]])
        # a shallow copy shares the grids, spectra, symbolic analysis and S-term map (which covers the base's
        # branches only); the branch list, numbering of the unknowns and the caches are its own
        new = copy.copy(root)
        new.top = t
        new.branches_all = new.branches = branches
        new.nbr, new.nb = t.nbr, t.nb
        new.full_label, new.cond_label = t.full_label, t.cond_label
        new.dense = layout.dense_layout(t)
        new.n_table = root.tab_br0 + t.nbr
        new.n_lowrank = t.nbr - root.nbr
        new._base = root
        new._moment_w = None
        new._lock = threading.Lock()
        new._ops = OrderedDict()
        new._device = root._device if device is None else bool(device) and root._device
        new.handle = native_geometry(new) if new._device else None
        return new

    def map_state(self, x: Optional[np.ndarray], stack: "PlaneStack") -> Optional[np.ndarray]:
        """A solution vector of `stack` in this stack's unknowns (a warm start), peec.py:1914-1923: the same
        stack, or one whose branches lead this one's on the same base, whose added branches start with zero
        current; None otherwise."""
        if x is None:
            return None
        if stack is self:
            return x
        root = self._base if self._base is not None else self
        sroot = stack._base if stack._base is not None else stack
        n = len(stack.branches)
        if sroot is root and n <= len(self.branches) and all(p is q for p, q in zip(stack.branches, self.branches)) \
                and len(x) == stack.nb + int(stack.keep.sum()):
            return np.concatenate([x[: stack.nb], np.zeros(self.nb - stack.nb, complex), x[stack.nb:]])
        return None

    # ------------------------------------------------------------------ per-frequency data
    def _freq_tables(self, f: float):
        """(omega, per operator the sheet impedances (S,) then the split layers' face couplings (n_twins,), cap
        impedances (npairs,), branch impedances (nbr,), admittance table (n_table,)) at f: peec.py:2150-2197 and
        2465-2511 restated over the table."""
        w = 2 * math.pi * f
        S, N = self.n_sheets, self.N
        zl = np.array([complex(greens.slab_impedance(l.thickness, f, self.sigma)) for l in self.layers])
        zsh = zl[self.sheet_layer]                         # a sheet's impedance per square
        zm = np.zeros(len(self.twin_parent), complex)
        if len(self.twin_parent):
            # a split layer's two faces: the face pair's own impedance and their coupling (peec.py:2161-2166)
            zself, zmut = greens.face_sheet_impedance(self.ts, f, self.sigma)
            for m, p in enumerate(self.twin_parent):
                zsh[p] = zsh[N + m] = zself[p]
                zm[m] = zmut[p]
        pl = self.top.pair_layers
        C = np.array([p.c_per_area for p in self.pairs]) * self.d ** 2
        tand = np.array([p.tan_delta for p in self.pairs])
        zcap = 1.0 / (w * C * tand + 1j * w * C) if w > 0 else np.full(len(pl), 1e18 + 0j)
        zbr = np.array([complex(b.z(f)) for b in self.branches], complex)
        if self.branch_scale is not None and len(zbr):   # a branch's resistance only (its inductance stays)
            zbr = zbr.real * self.branch_scale[: len(zbr)] + 1j * zbr.imag
        ncode = 1 << S
        tab = np.zeros(self.n_table, complex)
        z12 = {N + m: zm[m] for m in range(len(zm))}
        for o, name in enumerate("xy"):
            for code in range(1, ncode):
                lay = [k for k in range(S) if code >> k & 1]
                blk = self._dinv_block(name, lay, zsh[lay], np.zeros(len(lay)), z12, w)
                tab[(o * ncode + code) * S * S: (o * ncode + code + 1) * S * S] = blk.ravel()
        if self.n_override:
            self._override_blocks(tab, w, zsh, zm)
        tab[self.tab_cap0: self.tab_br0] = 1.0 / zcap if len(pl) else []
        tab[self.tab_br0:] = 1.0 / zbr if self.nbr else []
        return w, np.concatenate([zsh, zm]), zcap, zbr, tab

    def _override_blocks(self, tab: np.ndarray, w: float, zsh: np.ndarray, zm: np.ndarray):
        """D^-1 blocks of the positions whose strips are not all full squares (peec.py:2480-2509: each such
        position its own R / width and self inductance + dL, a face pair's coupling / width)."""
        t, S, N = self.top, self.n_sheets, self.N
        sidx = {}
        for name, idx, lo in (("x", t.xa, 0), ("y", t.ya, self.nxb)):
            a = -np.ones((S, *self.override[name].shape), np.int64)
            if len(idx):
                a[tuple(idx.T)] = lo + np.arange(len(idx))
            sidx[name] = a
        dL = self.dL if self.dL is not None else np.zeros(self.ns)
        for q, (o, i, j) in enumerate(self.override_pos):
            name = "xy"[o]
            strips = sidx[name][:, i, j]
            lay = [k for k in range(S) if strips[k] >= 0]
            st_ = strips[lay]
            sc = self.r_scale[st_] if self.r_scale is not None else np.ones(len(st_))
            R = (zsh[lay].real * sc + 1j * zsh[lay].imag) / self.r_width[st_]
            z12 = {}
            for k in lay:
                if k >= N:
                    sk = self.r_scale[strips[k]] if self.r_scale is not None else 1.0
                    z12[k] = (zm[k - N].real * sk + 1j * zm[k - N].imag) / self.r_width[strips[k]]
            blk = self._dinv_block(name, lay, R, dL[st_], z12, w)
            tab[self.tab_ovr0 + q * S * S: self.tab_ovr0 + (q + 1) * S * S] = blk.ravel()

    def set_resistance_scale(self, strips: Optional[np.ndarray] = None, branches: Optional[np.ndarray] = None):
        """Scale the strips' resistances (one factor per strip, x strips then y strips) and the branches' (their
        real part), e.g. by 1 + alpha (T - 20 C) for copper at its temperature; None: as built
        (peec.py:2199-2216).  The factorisations made before are dropped; the device geometry is rebuilt with
        the scaled strips' own preconditioner blocks and correction rows."""
        r = None if strips is None else np.asarray(strips, float)
        b = None if branches is None else np.asarray(branches, float)
        if r is not None and len(r) != self.ns:
            raise ValueError(f"{len(r)} strip factors for {self.ns} strips")
        if b is not None and len(b) != len(self.branches):
            raise ValueError(f"{len(b)} branch factors for {len(self.branches)} branches")
        if self._base is not None:
            raise ValueError("scale the base stack's resistances, then derive")
        with self._lock:
            self.r_scale, self.branch_scale = r, b
            self._corrections()
            self._schur_structure(self.leaf, sym=self.sym)
            self._ops.clear()
            if self._device:
                self.handle = native_geometry(self)

    def operator(self, f: float):
        """The device operator (factorised Schur complement) at f's key, made once and cached."""
        key = freq_key(f)
        with self._lock:
            op = self._ops.get(key)
            if op is not None:
                self._ops.move_to_end(key)
                return op
        op = self.factorise([key])[0]
        return op

    def factorise(self, freqs, together: bool = False, borrow: bool = False) -> list:
        """Factorise the Schur complement at each frequency key on the device (one batched launch per
        elimination level); returns the cached operators [(Operators, index)].  together: all of them in one
        Operators object (what a batched solve needs), refactorising cached ones that live elsewhere.
        borrow: let a frequency be preconditioned by a neighbouring one's factorisation (borrow_plan)."""
        from . import native
        keys = [freq_key(f) for f in freqs]
        if self._base is not None:
            return self._factorise_derived(keys, borrow)
        todo = [k for k in dict.fromkeys(keys) if k not in self._ops]
        if together and not todo and (len({id(self._ops[k][0]) for k in keys}) > 1 or
                                      any((self._ops[k][0].factor_of is not None) != borrow for k in keys)):
            todo = list(dict.fromkeys(keys))
        elif together and todo and len(todo) < len(set(keys)):
            todo = list(dict.fromkeys(keys))
        if todo:
            plan = borrow_plan(todo) if borrow else None
            self._admit(len(set(plan)) if plan is not None else len(todo))
            data = [self._freq_tables(k) for k in todo]
            ops = native.Operators(self.handle, todo, data, plan, fp32_panels=self.fp32_panels)
            ops.stiff = any(native.stiff_table(d[4], self.tab_cap0) for d in data)
            with self._lock:
                for n, k in enumerate(todo):
                    self._ops[k] = (ops, n)
                while len(self._ops) > max(OPERATOR_CACHE, len(keys)):
                    self._ops.popitem(last=False)
        return [self._ops[k] for k in keys]

    def _factorise_derived(self, keys: list, borrow: bool) -> list:
        """A derived stack's operators: its base's factorisations of the keys (made there if need be) with the
        low-rank update for the added branches (peec.py:2354-2377), one set per base operator set."""
        from . import native
        bops = self._base.factorise(keys, together=True, borrow=borrow)
        bobj = bops[0][0]
        with self._lock:
            cached = all(k in self._ops and self._ops[k][0].base is bobj for k in keys)
        if not cached:
            data = [self._freq_tables(k) for k in bobj.keys]
            dobj = native.Operators(self.handle, bobj.keys, data, base=bobj)
            dobj.stiff = any(native.stiff_table(d[4], self.tab_cap0) for d in data)
            with self._lock:
                for n, k in enumerate(bobj.keys):
                    self._ops[k] = (dobj, n)
                while len(self._ops) > max(OPERATOR_CACHE, len(keys)):
                    self._ops.popitem(last=False)
        return [self._ops[k] for k in keys]

    # ------------------------------------------------------------------ solves
    def solve(self, f: float, rhs_top: np.ndarray, J: np.ndarray, tol: float = 1e-5, max_cycles: int = 8,
              guess: Optional[list] = None):
        """Solve K [I; V] = [rhs_top; J] (peec.py:2513-2607).  Returns (Ib (nb), V (n_nodes), its, x).
        max_cycles is taken for the reference's signature: the reference restarts GMRES max_cycles times (and
        more while each restart still lowers the residual, peec.py:3093-3110); the device's FP64 outer
        iteration instead stops at tol, at max_its inner iterations (solve_batch) or after 40 outer steps."""
        out = self.solve_batch([f], [np.asarray(rhs_top, complex)], [np.asarray(J, float)], tol=tol,
                               max_cycles=max_cycles, guesses=[guess])
        return out[0]

    def rhs_vector(self, rhs_top: np.ndarray, J: np.ndarray) -> np.ndarray:
        return np.concatenate([np.asarray(rhs_top, complex), np.asarray(J, float)[self.keep].astype(complex)])

    def solve_batch(self, freqs, rhs_tops, Js, tol: float = 1e-5, max_cycles: int = 8, guesses=None,
                    restart: int = 50, max_its: int = 2000, inner_tol: float = 1e-5, precision: str = "mixed",
                    reorth: float = 0.7, borrow: bool = False, failed: Optional[list] = None):
        """Many columns (frequency, right-hand side) in one device run: returns [(Ib, V, its, x, residual)].
        A column that misses tol raises SolverError, or, when a list is passed as `failed`, has its index
        appended there (its entry holds the best solution found)."""
        from . import native
        ncol = len(freqs)
        ops = self.factorise(freqs, together=True, borrow=borrow)
        rhs = np.stack([self.rhs_vector(r, j) for r, j in zip(rhs_tops, Js)])
        x0 = self._warm_start(ops, rhs, guesses) if guesses is not None else None
        x = np.zeros_like(rhs)
        its, res, ok = np.zeros(ncol, np.int32), np.zeros(ncol), np.zeros(ncol, bool)
        if precision == "mixed" and any(getattr(o[0], "stiff", False) for o in ops):
            # a stiff factorisation (near-short branches): the library applies its preconditioner in FP64; plan
            # the memory for that
            precision = "mixed_pc64"
        step = self.columns_that_fit(ncol, restart, precision)
        for c0 in range(0, ncol, step):
            sl = slice(c0, c0 + step)
            x[sl], its[sl], res[sl], ok[sl] = native.solve(
                self.handle, ops[sl], rhs[sl], tol=tol, restart=restart, max_its=max_its, inner_tol=inner_tol,
                precision=precision, reorth=reorth, x0=None if x0 is None else x0[sl])
        lender = getattr(ops[0][0], "factor_of", None) if borrow else None
        lent = [c for c in range(ncol) if not ok[c] and lender is not None and lender[ops[c][1]] != ops[c][1]]
        if lent:
            # a borrowed preconditioner that did not get there: factorise at the columns' own frequencies and go
            # on from their solutions so far (peec.py:2584-2595)
            again = self.solve_batch([freqs[c] for c in lent], [rhs_tops[c] for c in lent], [Js[c] for c in lent],
                                     tol=tol, guesses=[[x[c]] for c in lent], restart=restart, max_its=max_its,
                                     inner_tol=inner_tol, precision=precision, reorth=reorth, borrow=False,
                                     failed=[])
            for c, r in zip(lent, again):
                x[c], its[c], res[c], ok[c] = r[3], its[c] + r[2], r[4], r[4] <= tol
        out = []
        for c in range(ncol):
            if not ok[c]:
                if failed is None:
                    raise SolverError(f"GMRES did not converge at {freqs[c]:.4g} Hz ({its[c]} iterations, "
                                      f"residual {res[c]:.3g})")
                failed.append(c)
            V = np.zeros(self.n_nodes, complex)
            V[self.keep] = x[c, self.nb:]
            out.append((x[c, : self.nb], V, int(its[c]), x[c], float(res[c])))
        return out

    MEMORY_HEADROOM = 0.9         # of the device's free memory a solve or a factorisation may take

    def factorisation_bytes(self, n_fact: int) -> int:
        """Device bytes of n_fact factorisations while they are made (gt_operators_create_ex): each one's panels in
        FP64 and FP32, column- and row-major (with fp32_panels the FP32 pair kept and the FP64 factor in
        temporary memory), its pivots and tables, and the Schur values and update matrices."""
        sym = self.sym
        panel = (16 + 8 + 8) if self.fp32_panels else (16 + 8 + 8 + 16)
        per = sym.panel_total * panel + sym.n * (16 + 8) + self.n_table * (16 + 8)
        made = self.sterm.shape[0] * 16 + max(sym.upd_total, 1) * 16
        return int(n_fact * (per + made))

    def resident_bytes(self, n_fact: int) -> int:
        """Device bytes n_fact factorisations hold once made."""
        sym = self.sym
        panel = (8 + 8) if self.fp32_panels else (16 + 8 + 8 + 16)
        return int(n_fact * (sym.panel_total * panel + sym.n * (16 + 8) + self.n_table * (16 + 8)))

    def trim(self):
        """Free the device solve workspace of this stack (the next solve makes it again)."""
        if self.handle is not None:
            self.handle.trim()

    def release_operators(self):
        """Drop this stack's cached factorisations (their device memory goes when nothing else holds them)."""
        with self._lock:
            self._ops.clear()

    def _admit(self, n_fact: int):
        """The memory gate for factorisations (_MemoryGate, peec.py:1442-1501): when n_fact more would not fit
        MEMORY_HEADROOM of the free device memory, this stack's cached factorisations are dropped first; still
        too little: MemoryError."""
        from . import native
        need = self.factorisation_bytes(n_fact)
        free = native.memory(self.handle, 1)["free"]
        if need <= self.MEMORY_HEADROOM * free:
            return
        with self._lock:
            self._ops.clear()
        import gc
        gc.collect()
        self.trim()                   # and the solve workspace, which the next solve makes again
        free = native.memory(self.handle, 1)["free"]
        if need > self.MEMORY_HEADROOM * free:
            raise MemoryError(f"{n_fact} factorisations need {need / 2**30:.1f} GiB, "
                              f"{self.MEMORY_HEADROOM * free / 2**30:.1f} GiB are available on the device")

    def columns_that_fit(self, ncol: int, restart: int = 50, precision: str = "mixed") -> int:
        """How many columns one device solve takes at once (the reference's memory gate, peec.py:1388-1501):
        all of them when their workspace fits the geometry's present one plus MEMORY_HEADROOM of the free
        memory, else as many as fit; MemoryError when not even one does."""
        from . import native
        full = native.memory(self.handle, ncol, restart, precision)
        room = full["held"] + self.MEMORY_HEADROOM * full["free"]
        if full["need"] <= room:
            return ncol
        one = native.memory(self.handle, 1, restart, precision)["need"]
        per = (full["need"] - one) / max(ncol - 1, 1)
        fit = int((room - one) // per) + 1 if room >= one else 0
        if fit < 1:
            raise MemoryError(f"a solve of one column needs {one / 2**30:.1f} GiB, "
                              f"{room / 2**30:.1f} GiB are available on the device")
        return min(fit, ncol)

    def _warm_start(self, ops, rhs: np.ndarray, guesses) -> Optional[np.ndarray]:
        """Starting points from guess vectors (peec.py:2570-2578): per column x0 = G c with c minimising
        ||K G c - b|| (the FP64 device products of every column's guess vectors in one batch), kept where it
        lowers the residual below 0.9 of ||b||; None when no column has one."""
        from . import native
        vecs, owner, idx = [], [], []
        for c, guess in enumerate(guesses):
            for g in (guess or []):
                if g is not None and len(g) == rhs.shape[1] and np.any(g):
                    vecs.append(np.asarray(g, complex))
                    owner.append(c)
                    idx.append(ops[c][1])
        if not vecs:
            return None
        obj = ops[0][0]
        KG_all = native.apply(self.handle, obj, "matvec", np.stack(vecs), np.array(idx, np.int32), "fp64")
        owner = np.array(owner)
        x0 = np.zeros_like(rhs)
        used = False
        for c in np.unique(owner):
            sel = np.flatnonzero(owner == c)
            KG = KG_all[sel].T
            coef, *_ = np.linalg.lstsq(KG, rhs[c], rcond=None)
            if np.linalg.norm(rhs[c] - KG @ coef) < 0.9 * np.linalg.norm(rhs[c]):
                x0[c] = np.stack([vecs[q] for q in sel], axis=1) @ coef
                used = True
        return x0 if used else None

    # ------------------------------------------------------------------ coupling to a signal path
    def strip_coupling(self, segments: np.ndarray) -> np.ndarray:
        """psi of every strip (peec.py:2615-2656): on the device for a device stack (gt_strip_coupling), the
        host restatement otherwise."""
        if self.handle is not None:
            return self.handle.strip_coupling(self.sheet_z, self.sheet_t, self.d, segments, self.ns)
        px, py = greens.strip_coupling(segments, [self.xa, self.ya], self.d, self.sheet_z, self.sheet_t)
        return np.concatenate([px, py])

    def branch_coupling(self, segments: np.ndarray, start: int = 0, branches: Optional[list] = None) -> np.ndarray:
        """psi of the branches from `start` on (or of `branches`): a via's barrel couples to the trace's
        vertical segments."""
        vert = [s for s in segments if abs(s[5] - s[2]) > 0 and np.linalg.norm(s[3:5] - s[0:2]) < 1e-12]
        brs = self.branches[start:] if branches is None else list(branches)
        out = np.zeros(len(brs))
        for n, b in enumerate(brs):
            if b.kind == "via" and vert:
                pa, pb = self.pos(b.a), self.pos(b.b)
                out[n] = sum(s[7] * greens.segment_mutual(s[0:3], s[3:6], pa, pb, b.radius) for s in vert)
        return out

    def pos(self, node) -> np.ndarray:
        k, i, j = node
        return np.array([i * self.d, j * self.d, self.zs[k]])

    def moment_weights(self) -> np.ndarray:
        """(3, nb): the plane's part of the moment as a linear map of the branch currents, m = W Ib (peec.py:
        2680-2700: each strip's 1/2 r x dl at its sheet's height, each capacitance's and lumped branch's)."""
        W = getattr(self, "_moment_w", None)
        if W is not None and W.shape[1] == self.nb:
            return W
        d = self.d
        W = np.zeros((3, self.nb))
        k, _, j = self.xa.T                         # each strip at its sheet's height
        W[1, : self.nxb] = 0.5 * self.sheet_z[k] * d
        W[2, : self.nxb] = -0.5 * (j * d) * d
        k, i, _ = self.ya.T
        W[0, self.nxb: self.ns] = -0.5 * self.sheet_z[k] * d
        W[2, self.nxb: self.ns] = 0.5 * (i * d) * d
        if self.ncap:
            cu = self.top.cap[:, :4].astype(int)
            x, y = cu[:, 2] * d, cu[:, 3] * d
            dz = self.zs[cu[:, 1]] - self.zs[cu[:, 0]]
            W[0, self.ns: self.ns + self.ncap] = 0.5 * y * dz
            W[1, self.ns: self.ns + self.ncap] = -0.5 * x * dz
        for n, b in enumerate(self.branches):
            W[:, self.ns + self.ncap + n] = 0.5 * np.cross(self.pos(b.a), self.pos(b.b))
        self._moment_w = W
        return W

    def moment(self, segments: np.ndarray, Ib: np.ndarray) -> np.ndarray:
        """m = 1/2 sum r x I dl over the closed loop (peec.py:2668-2700): the trace's segments, then the plane's
        part (moment_weights)."""
        m = np.zeros(3, complex)
        for s in segments:
            m += 0.5 * s[7] * np.cross(s[0:3], s[3:6])
        return m + self.moment_weights() @ Ib


class RouteExcitation:
    """A current loop on a PlaneStack: the known trace current plus the driver/receiver injections
    (peec.py:2703-2817)."""

    def __init__(self, stack: PlaneStack, trace: list, inject_driver=None, inject_receiver=None,
                 trace_thickness: float = 35e-6, strip_psi: Optional[np.ndarray] = None,
                 branch_psi: Optional[np.ndarray] = None, injections: Optional[list] = None,
                 _L_trace: Optional[float] = None):
        """strip_psi / branch_psi: the coupling of the same loop computed on another stack with the same strips
        (a derived stack: RouteExcitation.on), reused; branches beyond branch_psi are coupled here.  _L_trace:
        the trace's own inductance, when already known for the same trace."""
        self.stack = stack
        self.trace = trace
        self.trace_t = trace_thickness
        self.inject = (inject_driver, inject_receiver)
        self.extra = list(injections or [])
        self.segments = np.array([[*s.a, *s.b, s.width, s.i] for s in trace], float).reshape(-1, 8)
        terms = []
        if inject_driver is not None:
            terms.append((inject_driver, -1.0, "driver return node"))
        if inject_receiver is not None:
            terms.append((inject_receiver, 1.0, "receiver return node"))
        terms += [(node, float(a), f"current injection at {node}") for node, a in (injections or [])]
        if not terms:
            raise SolverError("no current is injected")
        ids = []
        for node, amps, what in terms:
            n = stack.node_id(node)
            if n < 0:
                raise SolverError(f"{what} is not on plane copper")
            ids.append((n, amps))
        bal: dict = {}
        for n, amps in ids:
            c = int(stack.full_label[n])
            bal[c] = bal.get(c, 0.0) + amps
        if any(abs(v) > 1e-9 for v in bal.values()):
            if inject_driver is not None and inject_receiver is not None and not injections:
                raise SolverError("receiver return node is not connected to the driver's return node")
            raise SolverError("the injected currents do not balance on every connected piece of copper")
        self.injections = ids
        self.strip_psi = stack.strip_coupling(self.segments) if strip_psi is None else strip_psi
        bp = np.zeros(0) if branch_psi is None else np.asarray(branch_psi, float)
        if len(bp) < stack.nbr:
            bp = np.concatenate([bp, stack.branch_coupling(self.segments, start=len(bp))])
        self.branch_psi = bp[: stack.nbr]
        self.psi = np.concatenate([self.strip_psi, np.zeros(stack.ncap), self.branch_psi])
        if _L_trace is not None:
            self.L_trace = _L_trace
        else:
            self.L_trace = greens.trace_self(self.segments, trace_thickness) if len(trace) else 0.0

    def on(self, stack: PlaneStack) -> "RouteExcitation":
        """The same loop on a derived stack (with_branches), its strip coupling and the trace's own inductance
        reused (peec.py:2771-2774)."""
        return RouteExcitation(stack, self.trace, *self.inject, self.trace_t, self.strip_psi, self.branch_psi,
                               self.extra, _L_trace=self.L_trace)

    def J(self) -> np.ndarray:
        J = np.zeros(self.stack.n_nodes)
        for n, amps in self.injections:
            J[n] += amps
        return J

    def rhs_top(self, f: float) -> np.ndarray:
        return -1j * 2 * math.pi * f * self.psi

    def solution(self, f: float, Ib: np.ndarray, V: np.ndarray, its: int, res: float = 0.0) -> Solution:
        st = self.stack
        w = 2 * math.pi * f
        I_x = np.zeros((st.N, st.nx - 1, st.ny), complex)
        I_y = np.zeros((st.N, st.nx, st.ny - 1), complex)
        # per layer: a split layer's two faces added (peec.py:2796-2803)
        np.add.at(I_x, tuple(st.layer_index("x").T), Ib[: st.nxb])
        np.add.at(I_y, tuple(st.layer_index("y").T), Ib[st.nxb: st.ns])
        Vg = np.zeros((st.N, st.nx, st.ny), complex)
        Vg[np.nonzero(st.node)] = V[: st.n_grid]
        v_inj = sum(a * V[n] for n, a in self.injections)
        Z = complex(greens.trace_resistance(self.segments, f, st.sigma, self.trace_t) + v_inj
                    + 1j * w * (self.L_trace + np.dot(self.psi, Ib)))
        return Solution(f, I_x, I_y, Vg, Ib[st.ns + st.ncap:].copy(), Z, st.moment(self.segments, Ib), its,
                        Ib[st.ns: st.ns + st.ncap].copy(), res,
                        np.stack([Ib[st.tw_a], Ib[st.tw_b]]) if len(st.tw_b) else None, st.W_x, st.W_y, st.A_cu)

    def solve(self, f: float, guess=None, tol: float = 1e-5) -> Solution:
        Ib, V, its, x = self.stack.solve(f, self.rhs_top(f), self.J(), tol=tol, guess=guess)[:4]
        return self.solution(f, Ib, V, its)


def MultiPlaneProblem(layers: list, trace: list, inject_driver: tuple, inject_receiver: tuple,
                      branches: Optional[list] = None, sigma: float = SIGMA_CU, trace_thickness: float = 35e-6,
                      capacitance: Optional[list] = None, _device: bool = True) -> RouteExcitation:
    """A one-off problem: a stack plus one route (peec.py:2820-2826)."""
    return RouteExcitation(PlaneStack(layers, branches, capacitance, sigma, _device=_device), trace, inject_driver,
                           inject_receiver, trace_thickness)


def PlaneProblem(grid: Grid, trace: list, inject_driver: tuple, inject_receiver: tuple,
                 branches: Optional[list] = None, cu_thickness: float = 35e-6, sigma: float = SIGMA_CU,
                 trace_thickness: float = 35e-6, _device: bool = True) -> RouteExcitation:
    """A single plane at z = 0 under a trace (peec.py:2829-2837); nodes may be (i, j) or (0, i, j)."""
    fix = lambda n: tuple(n) if len(n) == 3 else (0, *n)  # noqa: E731
    br = [Branch(fix(b.a), fix(b.b), b.z, b.name, b.kind, b.radius) for b in (branches or [])]
    return MultiPlaneProblem([PlaneLayer("plane", 0.0, grid, cu_thickness)], trace, fix(inject_driver),
                             fix(inject_receiver), br, sigma, trace_thickness, _device=_device)


def solve_many(excitations: list, freqs, tol: float = 1e-5, **kw) -> list:
    """Every (excitation, frequency) pair on one stack in one device batch: [[Solution per f] per excitation]."""
    st = excitations[0].stack
    cols = [(e, f) for e in excitations for f in freqs]
    out = st.solve_batch([f for _, f in cols], [e.rhs_top(f) for e, f in cols], [e.J() for e, _ in cols], tol=tol, **kw)
    sols = [e.solution(f, Ib, V, its, res) for (e, f), (Ib, V, its, x, res) in zip(cols, out)]
    n = len(freqs)
    return [sols[k * n:(k + 1) * n] for k in range(len(excitations))]


def from_board(board, _device: bool = True):
    """A PlaneStack and its RouteExcitations for a ``synth.Board`` (the workloads' boards)."""
    grids = [Grid(0.0, 0.0, board.d * 1e3, board.nx, board.ny, l.node, l.xb, l.yb, **(l.widths or {}),
                  fill=l.fill, area=l.area, label=l.label) for l in board.layers]
    layers = [PlaneLayer(l.name, l.z, g, l.thickness) for l, g in zip(board.layers, grids)]
    branches = [Branch(b.a, b.b, b.z, f"br{n}", b.kind, b.radius) for n, b in enumerate(board.branches)]
    pairs = [PlanePair(p.upper, p.lower, p.c_per_area, p.tan_delta) for p in board.pairs]
    st = PlaneStack(layers, branches, pairs, board.sigma, precond=board.precond, screen=board.screen,
                    _device=_device)
    routes = []
    for net in board.nets:
        trace = [TraceSegment(s[0:3].copy(), s[3:6].copy(), float(s[6]), float(s[7])) for s in net.segments]
        routes.append(RouteExcitation(st, trace, net.driver, net.receiver, net.trace_t))
    return st, routes
