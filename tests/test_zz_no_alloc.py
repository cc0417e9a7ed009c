"""gt_lp_product_noalloc: the L_p product for callers that may not allocate device memory while they compute
(a process whose device memory is budgeted up front, a caller that cannot take cudaMalloc's device-wide
synchronisation).  It must give what the allocating entry point (gt_apply, kind "lp", FP64) gives, call after
call, although every call reuses the same fixed scratch array.  Collected last so a failure here never hides
another test's result; it builds everything it needs itself, so it also runs alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from groundtruth_gb300 import native, stack as gs
from test_oracle_golden import load

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_lp_product_without_allocation_matches_the_allocating_entry_point():
    torch = pytest.importorskip("torch")
    z, board = load("small_pair")
    st, routes = gs.from_board(board)
    obj, k = st.factorise([float(board.freqs[0])])[0]
    lib = st.handle.lib
    ncomp, ns, n = st.handle.n_compact, st.ns, st.handle.n_dense
    rng = np.random.default_rng(11)
    for call in range(2):                        # two calls in a row share the scratch array
        x = np.zeros((2, ncomp), complex)
        x[:, :ns] = rng.standard_normal((2, ns)) + 1j * rng.standard_normal((2, ns))
        ref = native.apply(st.handle, obj, "lp", x, k, "fp64")[:, :ns]
        X = torch.zeros((2, n), dtype=torch.complex128, device="cuda")
        Y = torch.zeros_like(X)
        st.handle.to_dense(x, X.data_ptr())
        rc = lib.gt_lp_product_noalloc(st.handle.h, 2, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()), None)
        assert rc == native.GT_OK, lib.gt_last_error()
        torch.cuda.synchronize()
        got = st.handle.to_compact(Y.data_ptr(), 2)[:, :ns]
        assert rel(got, ref) < 1e-12, call


def test_more_columns_than_the_fixed_scratch_holds_are_refused():
    torch = pytest.importorskip("torch")
    z, board = load("small_pair")
    st, routes = gs.from_board(board)
    lib = st.handle.lib
    # the FFT grid of one column: the larger orientation's sheets x padded row length x rows (rows rounded up
    # to a multiple of 16)
    pad = lambda n: (n + 15) // 16 * 16  # noqa: E731
    per_col = 16 * max(st.n_sheets * st.P["x"][1] * pad(st.nx - 1), st.n_sheets * st.P["y"][1] * pad(st.nx))
    too_many = (32 << 20) // per_col + 1
    # real buffers of that many columns: the call must refuse them before any kernel runs
    X = torch.zeros((too_many, st.handle.n_dense), dtype=torch.complex128, device="cuda")
    Y = torch.zeros_like(X)
    rc = lib.gt_lp_product_noalloc(st.handle.h, too_many, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()), None)
    assert rc == native.GT_INVALID_ARGUMENT
    assert b"fewer columns" in lib.gt_last_error()
