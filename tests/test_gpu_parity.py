"""Parity of the CUDA path with the reference: device products against the reference's own products and
solves (golden fixtures), through the C ABI.  Needs a GPU."""
import numpy as np
import pytest

from groundtruth_gb300 import native, stack as gs
from test_oracle_golden import load

pytestmark = pytest.mark.gpu
CASES = ["small_pair", "small_stack3", "plain_plane", "necked_pair", "faces_stack3_diag", "faces_stack3_sheet",
         "necked_faces"]


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module", params=CASES)
def case(request):
    z, board = load(request.param)
    st, routes = gs.from_board(board)
    return request.param, z, board, st, routes


def _op(st, f):
    obj, k = st.factorise([f])[0]
    return obj, k


# FP64 products: rounding-level agreement with the reference (its FFT sizes differ from ours)
def test_fp64_system_product(case):
    name, z, board, st, routes = case
    obj, k = _op(st, float(z["op_f"]))
    y = native.apply(st.handle, obj, "matvec", z["prod_x"], k, "fp64")[0]
    assert rel(y, z["prod_matvec"]) < 1e-12


def test_fp64_lp_product(case):
    name, z, board, st, routes = case
    obj, k = _op(st, float(z["op_f"]))
    x = np.zeros(st.nb + int(st.keep.sum()), complex)
    x[: st.ns] = z["prod_I"]
    y = native.apply(st.handle, obj, "lp", x, k, "fp64")[0][: st.ns]
    assert rel(y, z["prod_Lp"]) < 1e-12


def test_fp64_preconditioner(case):
    name, z, board, st, routes = case
    obj, k = _op(st, float(z["op_f"]))
    y = native.apply(st.handle, obj, "precond", z["prod_x"], k, "fp64")[0]
    assert rel(y, z["prod_precond"]) < 1e-9


# FP32 products: within single-precision rounding of the FP64 reference
def test_fp32_system_product(case):
    name, z, board, st, routes = case
    obj, k = _op(st, float(z["op_f"]))
    y = native.apply(st.handle, obj, "matvec", z["prod_x"], k, "fp32")[0]
    assert rel(y, z["prod_matvec"]) < 2e-6


def test_fp32_preconditioner(case):
    name, z, board, st, routes = case
    obj, k = _op(st, float(z["op_f"]))
    y = native.apply(st.handle, obj, "precond", z["prod_x"], k, "fp32")[0]
    assert rel(y, z["prod_precond"]) < 1e-3


@pytest.mark.parametrize("precision", ["mixed", "mixed16", "fp64"])
def test_solves_match_reference(case, precision):
    """Every (net, frequency) of the fixture in one batch; rtol 1e-10 like the reference run.  Both stop at a
    backward error of 1e-10, so the solutions agree to within the conditioning times that."""
    name, z, board, st, routes = case
    sols = gs.solve_many(routes, list(board.freqs), tol=board.tol, precision=precision)
    for k, per in enumerate(sols):
        for q, sol in enumerate(per):
            x_ref = z[f"x{k}_{q}"]
            Ib = x_ref[: st.nb]
            assert rel(sol.state_for(st)[: st.ns], Ib[: st.ns]) < 1e-7, (k, q)
            Zr = complex(z[f"Z{k}_{q}"])
            assert abs(sol.Z_loop - Zr) <= 1e-8 * abs(Zr), (k, q, sol.Z_loop, Zr)
            assert rel(sol.m, z[f"m{k}_{q}"]) < 1e-7
            assert sol.residual <= board.tol


def test_warm_start_guess(case):
    """peec.py:2570-2578: a guess spanning the solution starts the solve there; a poor one is ignored."""
    name, z, board, st, routes = case
    f = float(board.freqs[0])
    r = routes[0]
    Ib, V, its, x = st.solve(f, r.rhs_top(f), r.J(), tol=board.tol)[:4]
    Ib2, V2, its2, x2 = st.solve(f, r.rhs_top(f), r.J(), tol=board.tol, guess=[x])[:4]
    assert its2 == 0 and rel(x2, x) < 1e-9
    rng = np.random.default_rng(3)
    noisy = x * (1 + 1e-3 * rng.standard_normal(len(x)))
    Ib3, V3, its3, x3 = st.solve(f, r.rhs_top(f), r.J(), tol=board.tol, guess=[noisy])[:4]
    assert its3 < its and rel(x3, x) < 1e-7
    junk = rng.standard_normal(len(x)) * np.linalg.norm(x)
    Ib4, V4, its4, x4 = st.solve(f, r.rhs_top(f), r.J(), tol=board.tol, guess=[junk])[:4]
    assert rel(x4, x) < 1e-7


def test_strip_coupling_on_device(case):
    """psi of every strip on the device against the reference's own (fixture) and the host restatement."""
    name, z, board, st, routes = case
    from groundtruth_gb300 import greens
    for k, net in enumerate(board.nets):
        dev = st.handle.strip_coupling(st.sheet_z, st.sheet_t, st.d, net.segments, st.ns)
        px, py = greens.strip_coupling(net.segments, [st.xa, st.ya], st.d, st.sheet_z, st.sheet_t)
        host = np.concatenate([px, py])
        assert rel(dev, host) < 1e-12, k
        if f"psi{k}" in z.files:
            assert rel(dev, z[f"psi{k}"][: st.ns]) < 1e-12, k


def test_outputs_on_device(case):
    """Node fields and the plane's moment from a dense device solution against the host formulas."""
    import torch
    name, z, board, st, routes = case
    f = float(board.freqs[0])
    r = routes[0]
    Ib, V, its, x = st.solve(f, r.rhs_top(f), r.J(), tol=board.tol)[:4]
    if st.n_sheets != st.N:
        # face sheets: the outputs sum each split layer's faces on the host; the device entries refuse them
        X = torch.zeros((1, st.handle.n_dense), dtype=torch.complex128, device="cuda")
        with pytest.raises(ValueError):
            st.handle.moment(1, X.data_ptr(), st.sheet_z, st.d)
        return
    X = torch.zeros((1, st.handle.n_dense), dtype=torch.complex128, device="cuda")
    st.handle.to_dense(x[None, :], X.data_ptr(), 0)
    kx = torch.zeros((1, st.N, st.nx, st.ny), dtype=torch.complex128, device="cuda")
    ky = torch.zeros_like(kx)
    st.handle.node_field(1, X.data_ptr(), st.d, kx.data_ptr(), ky.data_ptr())
    I_x = np.zeros((st.N, st.nx - 1, st.ny), complex)
    I_y = np.zeros((st.N, st.nx, st.ny - 1), complex)
    I_x[tuple(st.xa.T)] = Ib[: st.nxb]
    I_y[tuple(st.ya.T)] = Ib[st.nxb: st.ns]
    sol = gs.Solution(f, I_x, I_y, np.zeros((st.N, st.nx, st.ny), complex), Ib[st.ns + st.ncap:], 0j,
                      np.zeros(3, complex), its)
    for k in range(st.N):
        hx, hy = sol.node_field(k, st.d * 1e3)
        assert rel(kx[0, k].cpu().numpy(), hx) < 1e-13 and rel(ky[0, k].cpu().numpy(), hy) < 1e-13
    m_dev = st.handle.moment(1, X.data_ptr(), st.zs, st.d)[0]
    m_host = st.moment(np.zeros((0, 8)), Ib)
    assert rel(m_dev, m_host) < 1e-12


@pytest.mark.parametrize("shape", [(39, 36, 0.5e-3, 0.0), (39, 36, 0.5e-3, 0.2e-3), (255, 256, 0.25e-3, 1.07e-3),
                                   (29, 44, 0.4e-3, 0.335e-3)])
def test_kernel_spectrum_on_device(shape):
    """The strip kernel's spectrum quadrant on the device against the host FFT of the host kernel."""
    from groundtruth_gb300 import greens
    na, nl, d, dz = shape
    P0, P1 = greens.fft_size(2 * na - 1), greens.fft_size(2 * nl - 1)
    host = greens.spectrum_quadrant(greens.strip_kernel(na, nl, d, dz), P0, P1)
    dev = native.kernel_spectrum(na, nl, d, dz, P0, P1, greens.near_values(na, nl, d, dz))
    assert np.max(np.abs(dev - host)) <= 1e-12 * np.max(np.abs(host))


def test_solves_with_borrowed_preconditioners(case):
    """Every other frequency preconditioned by its neighbour's factorisation (gt_operators_create_shared): the
    same solutions, the system always at the column's own frequency."""
    name, z, board, st, routes = case
    freqs = list(board.freqs)
    if len(freqs) < 2 or gs.borrow_plan(freqs) == list(range(len(freqs))):
        freqs = [freqs[0], freqs[0] * 1.2]
    sols = gs.solve_many(routes, freqs, tol=board.tol, borrow=True)
    ref = gs.solve_many(routes, freqs, tol=board.tol)
    for per, per_ref in zip(sols, ref):
        for sol, r in zip(per, per_ref):
            assert sol.residual <= board.tol
            assert abs(sol.Z_loop - r.Z_loop) <= 1e-8 * abs(r.Z_loop)


@pytest.mark.parametrize("name", ["necked_pair_scaled", "faces_stack3_sheet_scaled"])
def test_resistance_scale_on_device(name):
    """PlaneStack.set_resistance_scale (peec.py:2199-2216) on the device: products, preconditioner and solves
    against the reference's scaled stack."""
    z, board = load(name)
    st, routes = gs.from_board(board)
    st.set_resistance_scale(z["r_scale"], z["branch_scale"])
    obj, k = _op(st, float(z["op_f"]))
    assert rel(native.apply(st.handle, obj, "matvec", z["prod_x"], k, "fp64")[0], z["prod_matvec"]) < 1e-12
    assert rel(native.apply(st.handle, obj, "precond", z["prod_x"], k, "fp64")[0], z["prod_precond"]) < 1e-9
    sols = gs.solve_many(routes, list(board.freqs), tol=board.tol)
    for kk, per in enumerate(sols):
        for q, sol in enumerate(per):
            Zr = complex(z[f"Z{kk}_{q}"])
            assert abs(sol.Z_loop - Zr) <= 1e-8 * abs(Zr), (kk, q)
            assert sol.residual <= board.tol


def test_memory_gate_counts_the_workspace(case):
    """gt_memory: a solve's bytes grow with its columns; after a solve the geometry's workspace holds what it
    said it would need (less the compact staging)."""
    name, z, board, st, routes = case
    m1, m4 = native.memory(st.handle, 1), native.memory(st.handle, 4)
    assert 0 < m1["need"] < m4["need"] and 0 < m4["free"] <= m4["total"]
    f = float(board.freqs[0])
    r = routes[0]
    st.solve_batch([f] * 4, [r.rhs_top(f)] * 4, [r.J()] * 4, tol=board.tol)
    held = native.memory(st.handle, 4)["held"]
    assert held >= m4["need"] - 4 * st.handle.n_compact * 16


@pytest.mark.parametrize("name", ["small_pair", "necked_faces"])
def test_not_converged_is_reported(name):
    """Forced non-convergence, an iteration limit of 2 against a tolerance of 1e-12 (peec.py:2599-2600): a
    SolverError naming the frequency, or, with `failed`, every column's index and its solution so far; the device
    state stays usable and the next solve at the board's tolerance converges."""
    z, board = load(name)
    st, routes = gs.from_board(board)
    r = routes[0]
    fs = [float(f) for f in board.freqs[:2]]
    args = (fs, [r.rhs_top(f) for f in fs], [r.J()] * len(fs))
    with pytest.raises(gs.SolverError, match="did not converge"):
        st.solve_batch(*args, tol=1e-12, max_its=2)
    failed = []
    out = st.solve_batch(*args, tol=1e-12, max_its=2, failed=failed)
    assert failed == list(range(len(fs)))
    assert all(np.isfinite(o[3]).all() and o[4] > 1e-12 for o in out)
    sol = gs.solve_many(routes[:1], fs[:1], tol=board.tol)[0][0]
    assert sol.residual <= board.tol
    assert abs(sol.Z_loop - complex(z["Z0_0"])) <= 1e-8 * abs(complex(z["Z0_0"]))


def test_repeated_solves_are_bit_identical():
    """The reference's determinism checks (a repeated run gives identical numbers: test_numerics_audit.py:245-251,
    test_speed.py:103-157): the same batch solved twice on one stack takes the same iterations and gives
    bit-identical currents, potentials and loop impedances (fixed launch order, reductions in a fixed order)."""
    z, board = load("small_pair")
    st, routes = gs.from_board(board)
    fs = [float(f) for f in board.freqs]
    first = gs.solve_many(routes, fs, tol=board.tol)
    again = gs.solve_many(routes, fs, tol=board.tol)
    for pa, pb in zip(first, again):
        for a, b in zip(pa, pb):
            assert a.iterations == b.iterations and a.Z_loop == b.Z_loop
            assert np.array_equal(a.I_x, b.I_x) and np.array_equal(a.I_y, b.I_y) and np.array_equal(a.V, b.V)
