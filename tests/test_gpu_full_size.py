"""Full-size parity of the plane currents: three columns of the 256 x 256 slotted plane pair (4-layer board, 8
nets x 32 frequencies; nets 0 / 1 / 0 at 1 MHz, 28.3 MHz and 1 GHz) solved through the CUDA library to rtol 1e-10,
against the reference's own FP64 solves of the same columns (tests/golden/slotted_pair_currents.npz, made by
make_golden.py --currents-only): the plane current maps I_x, I_y of both sheets within 1e-6 relative L2 and
Z_loop within 1e-8.  Needs a GPU."""
from pathlib import Path

import numpy as np
import pytest

from groundtruth_gb300 import stack as gs, synth

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden" / "slotted_pair_currents.npz"


def test_full_size_currents_match_reference():
    z = np.load(GOLD)
    board = synth.slotted_pair()
    assert np.allclose(board.freqs, z["freqs"], rtol=1e-12, atol=0)
    st, routes = gs.from_board(board)
    cols = [(int(k), int(q)) for k, q in z["cols"]]
    res = st.solve_batch([float(board.freqs[q]) for _, q in cols],
                         [routes[k].rhs_top(float(board.freqs[q])) for k, q in cols],
                         [routes[k].J() for k, _ in cols], tol=1e-10, restart=50, max_its=4000, reorth=0.0)
    for n, ((k, q), (Ib, V, its, x, r)) in enumerate(zip(cols, res)):
        sol = routes[k].solution(float(board.freqs[q]), Ib, V, its, r)
        got = np.concatenate([np.ravel(sol.I_x), np.ravel(sol.I_y)])
        ref = np.concatenate([np.ravel(z[f"Ix{n}"]), np.ravel(z[f"Iy{n}"])]).astype(np.complex128)
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < 1e-6, (k, q, err)
        Zr = complex(z[f"Z{n}"])
        assert abs(sol.Z_loop - Zr) <= 1e-8 * abs(Zr), (k, q, sol.Z_loop, Zr)
        assert r <= 1e-10
