"""A plane between two others screens one side's field from the other: the face sheets of a screened layer
(GroundTruth: PlaneStack._faces, peec.py:1658-1716), against the one-dimensional exact values of a stack of
conducting slabs, as the reference's own tests state them (tests/test_plane_screening.py:1-28, 152-203).

Each case is a plane line: layers 10 mm wide rasterised from their copper (raster.build_layer, 0.4 mm pitch,
sub-grid 4), the VDD layer fed along its whole first column and shorted to the GND layer(s) along its last, two
lengths, their difference the line's inductance per length alone:

  * GND / VDD / GND, 0.1 mm gaps, 70 um copper: the middle plane returns half its current on each face,
        L' = (mu0 d + Li(t) + Li(t/2)) / 2w,  Li(t) the one-face slab's internal inductance;
  * VDD / floating plane / GND, 0.2 mm gaps, 35 um copper: the floating plane's faces carry eddy currents,
        L' = (mu0 2d + 2 Li(t) + Im(2 (k/sigma) tanh(k t/2)) / omega) / w,  k = (1 + j)/delta,
    transparent at low frequency and screening at high.

The ratios L'(f) / L'(1 MHz) against the exact ones cancel the field's fringing past the strips' edges; solved
by the oracle and, marked gpu, through the CUDA library."""
import math

import numpy as np
import pytest

from groundtruth_gb300 import raster, stack as gs
from oracle import peec_oracle as po

MU0, SIGMA = 4e-7 * math.pi, 5.8e7
W, PITCH = 10.0, 0.4
FREQS = (1e4, 1e6, 3e7, 1e8)


def _layers(stack, gaps, length):
    """[(name, z m, grid, t m)] top down: each layer's copper a box length x W mm, rasterised."""
    out, z = [], 0.0
    box = (np.array([[0.0, 0.0], [length, 0.0], [length, W], [0.0, W]]), [])
    for k, (net, t) in enumerate(stack):
        if k:
            z -= (0.5 * stack[k - 1][1] + gaps[k - 1] + 0.5 * t) * 1e-3
        g = raster.build_layer({net: [box]}, (0.0, 0.0, length, W), PITCH, sub=4)
        out.append((net, z, g, t * 1e-3))
    return out


def _ends(stack, g):
    """The shorts at the far end (VDD to every GND, 1 nOhm per node), the GND layers joined at the feed, and the
    feed: 1/ny A into VDD's and out of the first GND's first column."""
    nx, ny = g.nx, g.ny
    vdd = [k for k, (n, _) in enumerate(stack) if n == "VDD"][0]
    gnd = [k for k, (n, _) in enumerate(stack) if n == "GND"]
    shorts = [((vdd, nx - 1, j), (k, nx - 1, j)) for j in range(ny) for k in gnd]
    shorts += [((gnd[0], 0, j), (k, 0, j)) for j in range(ny) for k in gnd[1:]]
    feed = [((vdd, 0, j), 1.0 / ny) for j in range(ny)] + [((gnd[0], 0, j), -1.0 / ny) for j in range(ny)]
    return shorts, feed


def _oracle_line(stack, gaps, length):
    layers = _layers(stack, gaps, length)
    g = layers[0][2]
    shorts, feed = _ends(stack, g)
    st = po.OracleStack([po.OLayer(z, t, l.node, l.xb, l.yb, l.widths(), l.fill) for _, z, l, t in layers],
                        PITCH * 1e-3, [po.OBranch(a, b, 1e-9, 0.0) for a, b in shorts], screen=True)
    J = np.zeros(st.n_nodes)
    for node, amps in feed:
        J[st.nid[node]] += amps
    out = {}
    for f in FREQS:
        Ib, V, its, x = st.solve(f, np.zeros(st.nb, complex), J, tol=1e-5)
        out[f] = complex(sum(amps * V[st.nid[node]] for node, amps in feed))
    return out


def _device_line(stack, gaps, length):
    layers = _layers(stack, gaps, length)
    g = layers[0][2]
    shorts, feed = _ends(stack, g)
    grid = lambda l: gs.Grid(0.0, 0.0, PITCH, l.nx, l.ny, l.node, l.xb, l.yb, **l.widths(), fill=l.fill,  # noqa: E731
                             area=l.area)
    st = gs.PlaneStack([gs.PlaneLayer(n, z, grid(l), t) for n, z, l, t in layers],
                       [gs.Branch(a, b, lambda f: 1e-9 + 0j) for a, b in shorts], screen=True)
    route = gs.RouteExcitation(st, [], injections=feed)
    return {f: s.Z_loop for f, s in zip(FREQS, gs.solve_many([route], list(FREQS), tol=1e-5)[0])}


def _per_length(line, stack, gaps):
    a, b = line(stack, gaps, 20.0), line(stack, gaps, 40.0)
    return {f: ((b[f] - a[f]).imag / (2 * math.pi * f)) / 20e-3 for f in FREQS}


def _li(t, f):
    """The one-face slab's internal inductance per square: Im((1+j)/(sigma delta) coth((1+j) t/delta)) / omega."""
    delta = 1 / math.sqrt(math.pi * f * MU0 * SIGMA)
    u = (1 + 1j) * t / delta
    return (u * (1 + np.exp(-2 * u)) / (1 - np.exp(-2 * u)) / (SIGMA * t)).imag / (2 * math.pi * f)


def _eddy(t, f):
    """The floating slab's mode: Im(2 (k/sigma) tanh(k t/2)) / omega per square."""
    k = (1 + 1j) * math.sqrt(math.pi * f * MU0 * SIGMA)
    return (2 * k / SIGMA * np.tanh(k * t / 2)).imag / (2 * math.pi * f)


LINES = [pytest.param(_oracle_line, id="oracle"), pytest.param(_device_line, id="gpu", marks=pytest.mark.gpu)]


@pytest.mark.parametrize("line", LINES)
def test_a_plane_between_two_others_returns_on_both_faces(line):
    """GND / VDD / GND: L'(f) / L'(1 MHz) within 1 % of the exact ratio from 10 kHz to 100 MHz, L' within -3 / +5 %
    of the exact (one-dimensional) value."""
    per = _per_length(line, [("GND", 0.07), ("VDD", 0.07), ("GND", 0.07)], [0.1, 0.1])
    exact = {f: (MU0 * 0.1e-3 + _li(70e-6, f) + _li(35e-6, f)) / (2 * W * 1e-3) for f in FREQS}
    for f in FREQS:
        assert abs((per[f] / per[1e6]) / (exact[f] / exact[1e6]) - 1) < 0.01, f
        assert 0.97 < per[f] / exact[f] < 1.05, f


@pytest.mark.parametrize("line", LINES)
def test_a_floating_plane_screens_at_high_frequency_and_lets_the_field_through_at_low(line):
    """VDD / floating / GND against the same stack without the floating plane: the exact ratio within 1 % at every
    frequency, 1 within 1e-3 at 10 kHz (transparent), below 0.965 at 30 MHz (its faces' eddy currents)."""
    per = _per_length(line, [("VDD", 0.035), ("AUX", 0.035), ("GND", 0.035)], [0.2, 0.2])
    none = _per_length(line, [("VDD", 0.035), ("GND", 0.035)], [0.435])
    for f in FREQS:
        exact = (MU0 * 0.4e-3 + 2 * _li(35e-6, f) + _eddy(35e-6, f)) / (MU0 * 0.435e-3 + 2 * _li(35e-6, f))
        assert abs((per[f] / none[f]) / exact - 1) < 0.01, f
    assert abs(per[1e4] / none[1e4] - 1) < 1e-3
    assert per[3e7] / none[3e7] < 0.965


def _six_planes(screen: bool, d: float = 2.0):
    """Six planes (GND / VDD alternating, 35 um copper, 0.1 / 0.535 / 0.1 / 0.535 / 0.1 mm of dielectric) 24 x 16 mm
    on d mm cells (the grid cut at the board's edge: edge strips narrower than the pitch), the plane pairs'
    capacitance, VDD shorted to GND at one end and fed at the other ('sheet' preconditioner), on the oracle:
    (OracleStack, J)."""
    names = ["GND", "VDD", "GND", "VDD", "GND", "VDD"]
    gaps = [0.1, 0.535, 0.1, 0.535, 0.1]
    t, length, width = 0.035, 24.0, 16.0
    box = (np.array([[0.0, 0.0], [length, 0.0], [length, width], [0.0, width]]), [])
    layers, z = [], 0.0
    for k, net in enumerate(names):
        if k:
            z -= (t + gaps[k - 1]) * 1e-3
        g = raster.build_layer({net: [box]}, (0.0, 0.0, length, width), d, sub=4)
        layers.append(po.OLayer(z, t * 1e-3, g.node, g.xb, g.yb, g.widths(), g.fill))
    nx, ny = g.nx, g.ny
    vdd = [k for k, n in enumerate(names) if n == "VDD"]
    gnd = [k for k, n in enumerate(names) if n == "GND"]
    ends = [((vdd[0], nx - 1, j), (k, nx - 1, j)) for j in range(ny) for k in gnd]
    ends += [((vdd[0], 0, j), (k, 0, j)) for j in range(ny) for k in vdd[1:]]
    ends += [((gnd[0], 0, j), (k, 0, j)) for j in range(ny) for k in gnd[1:]]
    pairs = [po.OPair(k, k + 1, 8.854e-12 * 4.3 / (gaps[k] * 1e-3), 0.02) for k in range(5)]
    st = po.OracleStack(layers, d * 1e-3, [po.OBranch(a, b, 1e-9, 0.0) for a, b in ends], pairs, precond="sheet",
                        screen=screen)
    J = np.zeros(st.n_nodes)
    for j in range(ny):
        J[st.nid[(vdd[0], 0, j)]] += 1.0 / ny
        J[st.nid[(gnd[0], 0, j)]] -= 1.0 / ny
    return st, J


def test_the_face_pairs_difference_inductance_stays_positive_beside_narrow_strips():
    """test_plane_screening.py:256-276: a split layer's two faces share the narrow-strip corrections, so the
    difference mode (the free space between the faces, about mu0 t / 2 per face) stays positive definite at 15-25
    pH per square and the whole partial-inductance matrix with it."""
    st, _ = _six_planes(True)
    assert len(st.tw_b) and st.dL is not None and np.any(st.dL != 0)
    L = np.stack([st.Lp_matvec(np.eye(st.ns)[i].astype(complex)).real for i in range(st.ns)], axis=1)
    a, b = st.tw_a, st.tw_b
    assert abs(L - L.T).max() < 1e-12 * abs(L).max()
    diff = 0.5 * (L[np.ix_(a, a)] + L[np.ix_(b, b)] - L[np.ix_(a, b)] - L[np.ix_(b, a)])
    w = np.linalg.eigvalsh(diff)
    assert 15e-12 < w.min() and w.max() < 25e-12, (w.min(), w.max())
    assert np.linalg.eigvalsh(L).min() > 0.0


def test_a_split_stack_needs_about_the_iterations_of_the_unsplit_one():
    """test_plane_screening.py:279-288: the 'sheet' preconditioner on the six planes with and without face sheets
    takes within 1.3 x the iterations (GMRES to 1e-5) at 20, 100 and 400 MHz."""
    split, Js = _six_planes(True)
    plain, Jp = _six_planes(False)
    assert split.n_sheets == 10 and plain.n_sheets == 6
    for f in (2e7, 1e8, 4e8):
        its_s = split.solve(f, np.zeros(split.nb, complex), Js, tol=1e-5)[2]
        its_p = plain.solve(f, np.zeros(plain.nb, complex), Jp, tol=1e-5)[2]
        assert its_s <= 1.3 * its_p + 1, (f, its_s, its_p)


def _mean_log(w: float, ya: tuple, yb: tuple, n: int = 24) -> float:
    """The mean of ln r between two rectangles [0, w] x ya and [0, w] x yb (the geometric mean distance's log,
    Grover 1946): across the width in closed form, int int ln |x1 - x2, dy| dx1 dx2 / w^2 = (2/w^2) int_0^w
    (w - u) ln sqrt(u^2 + dy^2) du, and Gauss-Legendre over the two heights."""
    def across(dy: float) -> float:
        a = abs(dy)

        def prim(u: float) -> float:
            if a == 0.0:
                lu = math.log(u) if u > 0 else 0.0
                return w * (u * lu - u) - (0.5 * u * u * lu - 0.25 * u * u)
            lg = math.log(u * u + a * a)
            return w * 0.5 * (u * lg - 2 * u + 2 * a * math.atan(u / a)) - 0.25 * ((u * u + a * a) * lg - u * u)
        return 2.0 * (prim(w) - prim(0.0)) / (w * w)
    x, wt = np.polynomial.legendre.leggauss(n)
    pa = 0.5 * (ya[1] - ya[0]) * (x + 1) + ya[0]
    pb = 0.5 * (yb[1] - yb[0]) * (x + 1) + yb[0]
    return float(sum(wi * wj * across(p - q) for p, wi in zip(pa, wt) for q, wj in zip(pb, wt)) / 4.0)


def test_a_thin_dielectric_pair_converges_to_the_dc_distribution_with_the_cell_size():
    """test_plane_screening.py:206-225: 25 um of dielectric between 35 um copper, 10 mm wide, at 10 kHz (the DC
    current distribution): the line's inductance per length against two uniform plates' exact value,
    mu0 / 2 pi (2 ln g12 - ln g11 - ln g22), converges with the cell size: above it by under 11 % at 0.4 mm cells
    and under 4.5 % at 0.2 mm (first order: the cells' edge strips)."""
    global PITCH
    w, h, t = W * 1e-3, 25e-6, 35e-6
    exact = MU0 / (2 * math.pi) * (2 * _mean_log(w, (0, t), (t + h, 2 * t + h)) - 2 * _mean_log(w, (0, t), (0, t)))
    excess = []
    for pitch in (0.4, 0.2):
        old, PITCH = PITCH, pitch
        try:
            per = _per_length(_oracle_line, [("VDD", 0.035), ("GND", 0.035)], [0.025])
        finally:
            PITCH = old
        excess.append(per[1e4] / exact - 1)
    assert 0.0 < excess[0] < 0.11 and 0.0 < excess[1] < 0.045, excess
    assert excess[1] < 0.5 * excess[0] + 0.01, excess


def test_near_shorts_make_the_factorisation_stiff_and_ordinary_boards_do_not():
    """The 1 nOhm shorts of the GND / VDD / GND line put branch admittances of 1e9 S beside strips of a few
    hundred siemens: FP32 node potentials cannot resolve the volts across them, so the library applies that
    factorisation's preconditioner in FP64 (native.stiff_table is its rule).  A board of ordinary vias and
    parts stays on the FP32 preconditioner."""
    from groundtruth_gb300 import native, synth
    layers = _layers([("GND", 0.07), ("VDD", 0.07), ("GND", 0.07)], [0.1, 0.1], 20.0)
    g = layers[0][2]
    shorts, _ = _ends([("GND", 0.07), ("VDD", 0.07), ("GND", 0.07)], g)
    grid = lambda l: gs.Grid(0.0, 0.0, PITCH, l.nx, l.ny, l.node, l.xb, l.yb, **l.widths(), fill=l.fill,  # noqa: E731
                             area=l.area)
    st = gs.PlaneStack([gs.PlaneLayer(n, z, grid(l), t) for n, z, l, t in layers],
                       [gs.Branch(a, b, lambda f: 1e-9 + 0j) for a, b in shorts], screen=True, _device=False)
    for f in FREQS:
        assert native.stiff_table(st._freq_tables(f)[4], st.tab_cap0), f
    plain, _ = gs.from_board(synth.small_pair(), _device=False)
    for f in synth.small_pair().freqs:
        assert not native.stiff_table(plain._freq_tables(float(f))[4], plain.tab_cap0), f
