"""Pass C of the FP32 L_p product with its FFT-grid tiles brought in by TMA (lp.cu, lp_pass_ct) against the
same pass with per-warp 16-byte loads (lp_pass_cw, GT_LP_TMA=0): the same values in the same order, so the
products and the solves built on them agree bit for bit; and the product against the FP64 one.  The bench
board (256 x 256, 512-point rows) is the smallest that takes the 512-point warp passes.  Needs a GPU."""
import numpy as np
import pytest

from groundtruth_gb300 import native, stack as gs, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bench_board():
    b = synth.slotted_pair(n_nets=2, n_freq=3)
    st, routes = gs.from_board(b)
    assert st.P["x"][1] == 512 and st.P["y"][1] == 512
    return b, st, routes


def test_tma_tiles_give_the_products_of_the_plain_loads(bench_board, monkeypatch):
    b, st, routes = bench_board
    obj, k = st.factorise([float(b.freqs[1])])[0]
    rng = np.random.default_rng(5)
    n = st.handle.n_compact
    x = np.zeros((3, n), complex)
    x[:, : st.ns] = rng.standard_normal((3, st.ns)) + 1j * rng.standard_normal((3, st.ns))
    got = {}
    for flag in ("1", "0"):
        monkeypatch.setenv("GT_LP_TMA", flag)
        got[flag] = native.apply(st.handle, obj, "lp", x, k, "fp32")
    assert np.array_equal(got["1"], got["0"])
    ref = native.apply(st.handle, obj, "lp", x, k, "fp64")
    assert np.linalg.norm(got["1"] - ref) <= 1e-5 * np.linalg.norm(ref)


def test_tma_tiles_give_the_solves_of_the_plain_loads(bench_board, monkeypatch):
    b, st, routes = bench_board
    freqs = [float(f) for f in b.freqs]
    out = {}
    for flag in ("1", "0"):
        monkeypatch.setenv("GT_LP_TMA", flag)
        out[flag] = st.solve_batch(freqs, [routes[0].rhs_top(f) for f in freqs], [routes[0].J()] * len(freqs),
                                   tol=1e-10, reorth=0.0)
    for a, c in zip(out["1"], out["0"]):
        assert a[2] == c[2] and np.array_equal(a[3], c[3])
        assert a[4] <= 1e-10


def test_a_tma_wait_that_runs_out_is_reported_and_the_device_stays_usable(bench_board, monkeypatch):
    """Failure detection without a fault: the barrier is told to expect 16 bytes more than the two tile loads
    bring (GT_LP_TMA_TEST_SHORTFALL, with a 1 ms wait limit), so every block's wait runs out; the product
    returns GT_TIMEOUT (RuntimeError here), and the next product on the same context is right."""
    b, st, routes = bench_board
    obj, k = st.factorise([float(b.freqs[0])])[0]
    rng = np.random.default_rng(6)
    x = np.zeros((2, st.handle.n_compact), complex)
    x[:, : st.ns] = rng.standard_normal((2, st.ns)) + 1j * rng.standard_normal((2, st.ns))
    monkeypatch.setenv("GT_LP_TMA", "1")
    monkeypatch.setenv("GT_LP_TMA_TEST_SHORTFALL", "1")
    with pytest.raises(RuntimeError, match="did not arrive"):
        native.apply(st.handle, obj, "lp", x, k, "fp32")
    monkeypatch.delenv("GT_LP_TMA_TEST_SHORTFALL")
    got = native.apply(st.handle, obj, "lp", x, k, "fp32")
    ref = native.apply(st.handle, obj, "lp", x, k, "fp64")
    assert np.linalg.norm(got - ref) <= 1e-5 * np.linalg.norm(ref)
