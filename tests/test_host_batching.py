"""Host logic of the batch and serving drivers and of the pipelined sweep, without a GPU: the device-memory
budget's counting, the rule that sends an edit to a derived stack, and the sweep's column order check."""
import threading
import time
from types import SimpleNamespace

import numpy as np
import pytest

from groundtruth_gb300 import batch, native, serve, stack as gs, synth


def test_memory_budget_admits_what_fits_and_a_board_larger_than_it_alone():
    b = batch.MemoryBudget(10)
    assert b.acquire(6) == 6
    got = []

    def second():
        got.append(b.acquire(6))          # waits for the first release
    th = threading.Thread(target=second)
    th.start()
    time.sleep(0.1)
    assert not got
    b.release(6)
    th.join(2)
    assert got == [6]
    b.release(6)
    assert b.acquire(25) == 10            # larger than the whole budget: runs alone, within it
    b.release(10)
    assert b.used == 0


def test_an_edit_goes_to_the_derived_stack_only_when_it_joins_separate_copper():
    # one plane cut in two by a gap across the board: two pieces of copper, no capacitance between them
    n, d, t = 32, 0.5e-3, 35e-6
    gap = np.array([[15.4 * d, -d], [16.6 * d, -d], [16.6 * d, n * d], [15.4 * d, n * d]])
    layer = synth._full_layer("GND", 0.0, t, n, n, d, [gap])
    net = synth.Net(synth._segments([(4 * d, 8 * d), (12 * d, 8 * d)], 0.2e-3 + t, 0.5 * t, 0.2e-3), (0, 4, 8), (0, 12, 8))
    board = synth.Board("split", d, n, n, [layer], nets=[net], freqs=np.array([1e6]))
    st, _ = gs.from_board(board, _device=False)
    wi = SimpleNamespace(stack=st)
    on = [(k, i, j) for k in range(1) for i in range(board.nx) for j in range(board.ny) if st.node_id((k, i, j)) >= 0]
    lab = {n: int(st.full_label[st.node_id(n)]) for n in on}
    a = on[0]
    b = next(n for n in on if n != a and lab[n] == lab[a])
    c = next(n for n in on if lab[n] != lab[a])
    z = lambda f: 1e-3 + 0j
    same = serve.Request(nets=[0], freqs=[1e6], branches=[gs.Branch(a, b, z)])
    joins = serve.Request(nets=[0], freqs=[1e6], branches=[gs.Branch(a, c, z)])
    off = serve.Request(nets=[0], freqs=[1e6], branches=[gs.Branch(a, (0, -1, 0), z)])
    empty = serve.Request(nets=[0], freqs=[1e6])
    assert not serve.Server._joins(wi, same)
    assert serve.Server._joins(wi, joins)
    assert serve.Server._joins(wi, off)
    assert serve.Server._joins(wi, empty)


def test_a_sweep_wants_its_columns_sorted_by_frequency_group():
    keys = [1e6, 1e7, 1e8, 1e9]
    col_key = np.array([0, 0, 3, 1])           # a column of group 1 after one of group 3 (two groups of two)
    with pytest.raises(ValueError, match="sorted"):
        native.solve_sweep(None, keys, [None] * 4, col_key, np.zeros((4, 3), complex), 1e-10, chunks=2)
