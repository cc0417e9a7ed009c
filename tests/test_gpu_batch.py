"""Uneven boards solved side by side (groundtruth_gb300.batch): each board's solutions, iteration counts and loop
impedances are the same when it is solved alone and when it shares the device with others on their own streams,
and every column meets its tolerance.  Needs a GPU."""
import numpy as np
import pytest

from groundtruth_gb300 import batch, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def jobs():
    boards = [synth.random_board(s, side=(24, 64), n_layers=(2, 5), n_nets=(1, 3), n_freq=(2, 4)) for s in
              (41, 42, 43, 44, 45)]
    return batch.prepare(boards)


def test_a_board_solves_the_same_alone_and_in_the_mix(jobs):
    alone = [batch.solve_all([j], concurrency=1)[0] for j in jobs]
    mixed = batch.solve_all(jobs, concurrency=4)
    for a, m, j in zip(alone, mixed, jobs):
        assert a.name == m.name == j.name
        assert np.array_equal(a.its, m.its), j.name
        assert np.linalg.norm(a.x - m.x) <= 1e-12 * np.linalg.norm(a.x), j.name
        assert np.allclose(a.Z, m.Z, rtol=1e-12, atol=0), j.name
        assert np.all(m.residual <= j.tol), (j.name, m.residual.max())


def test_a_budget_smaller_than_one_board_runs_the_boards_one_at_a_time(jobs):
    small = batch.solve_all(jobs[:3], concurrency=3, budget_bytes=1)
    ref = [batch.solve_all([j], concurrency=1)[0] for j in jobs[:3]]
    for a, b in zip(small, ref):
        assert np.linalg.norm(a.x - b.x) <= 1e-12 * np.linalg.norm(b.x)


def _columns(st, routes, freqs, precision="mixed"):
    return st.solve_batch(freqs, [routes[0].rhs_top(f) for f in freqs], [routes[0].J()] * len(freqs), tol=1e-10,
                          precision=precision, reorth=0.0)


def test_operators_with_fp32_panels_only_solve_the_same_and_refuse_fp64():
    """FP32-panel operators (a third of the factor's memory) give the mixed solve the same panels, so the same
    answers bit for bit; an FP64 solve on them is refused with a clear error."""
    from groundtruth_gb300 import stack as gs
    b = synth.small_pair()
    st, routes = gs.from_board(b)
    freqs = [float(f) for f in b.freqs]
    ref = _columns(st, routes, freqs)
    st.release_operators()
    st.fp32_panels = True
    got = _columns(st, routes, freqs)
    for a, c in zip(ref, got):
        assert np.array_equal(a[3], c[3])
    with pytest.raises(ValueError, match="FP64 panels"):
        _columns(st, routes, freqs, precision="fp64")


@pytest.mark.parametrize("width", ["4", "2", "1"])
def test_narrow_column_groups_give_the_same_solutions(width, monkeypatch):
    """Fronts too wide for 8 columns' staging take groups of 4 or 2 (the panel read once per fewer columns):
    the same board solved with the group width capped equals its solve with groups of 8."""
    from groundtruth_gb300 import stack as gs
    b = synth.small_stack3()
    st, routes = gs.from_board(b)
    freqs = [float(f) for f in b.freqs] * 3           # more columns per operator than a group holds
    ref = _columns(st, routes, freqs)
    monkeypatch.setenv("GT_GROUP_WIDTH", width)
    got = _columns(st, routes, freqs)
    for a, c in zip(ref, got):
        assert np.linalg.norm(a[3] - c[3]) <= 1e-12 * np.linalg.norm(a[3])


def test_a_column_solves_the_same_in_any_batch():
    """A column's device arithmetic is its own: solved with every other column of the board, or alone, its
    iterations and solution are the same bit for bit (the triangular sweeps' partial sums meet in an order set
    by the fronts, not by how many columns share the launch)."""
    from groundtruth_gb300 import stack as gs
    b = synth.random_board(45, side=(24, 64), n_layers=(2, 5), n_nets=(1, 3), n_freq=(2, 4))
    st, routes = gs.from_board(b)
    freqs = [float(f) for f in b.freqs] * 4                 # enough columns for the many-task launch shapes
    together = _columns(st, routes, freqs)
    for q, f in enumerate(freqs[: len(b.freqs)]):
        alone = _columns(st, routes, [f])[0]
        assert alone[2] == together[q][2]                   # iterations
        assert np.array_equal(alone[3], together[q][3])     # solution


@pytest.mark.parametrize("chunks", [2, 3])
def test_a_sweep_factorised_beside_its_solves_equals_the_plain_solve(chunks):
    """native.solve_sweep (later frequency groups factorised on a second thread and stream while earlier ones
    solve) gives the plain path's results bit for bit: the same factorisations, and columns whose arithmetic
    does not depend on the batch they are solved in."""
    from groundtruth_gb300 import native, stack as gs
    b = synth.small_stack3()
    st, routes = gs.from_board(b)
    freqs = [float(f) for f in np.geomspace(1e6, 1e9, 6)]
    cols = [(k, q) for q in range(len(freqs)) for k in range(len(routes))]
    rhs = np.stack([st.rhs_vector(routes[k].rhs_top(freqs[q]), routes[k].J()) for k, q in cols])
    data = [st._freq_tables(f) for f in freqs]
    key = np.array([q for _, q in cols])
    ops = native.Operators(st.handle, freqs, data)
    x0, its0, res0, ok0 = native.solve(st.handle, [(ops, int(q)) for q in key], rhs, 1e-10, reorth=0.0)
    x1, its1, res1, ok1 = native.solve_sweep(st.handle, freqs, data, key, rhs, 1e-10, chunks=chunks, reorth=0.0)
    assert ok0.all() and ok1.all()
    assert np.array_equal(its0, its1)
    assert np.array_equal(x0, x1)
