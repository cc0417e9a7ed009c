"""layout.update_slots: the fronts' update matrices share storage only when their level spans do not meet (a
matrix is written at its front's level and read at its parent's), and the storage is a fraction of the sum."""
import numpy as np
import pytest

from groundtruth_gb300 import layout, stack as gs, synth


def _check(height, parent, size, off, total):
    end = np.where(parent >= 0, height[np.maximum(parent, 0)], height)
    for h in range(int(height.max()) + 1):
        live = [f for f in range(len(size)) if size[f] > 0 and height[f] <= h <= end[f]]
        spans = sorted((int(off[f]), int(off[f] + size[f])) for f in live)
        for (a0, a1), (b0, b1) in zip(spans, spans[1:]):
            assert a1 <= b0, (h, (a0, a1), (b0, b1))
        assert all(0 <= a and b <= total for a, b in spans)


@pytest.mark.parametrize("make", [synth.small_pair, synth.small_stack3, lambda: synth.random_board(31),
                                  lambda: synth.largest_board(48, n_nets=1, n_freq=1)])
def test_live_update_matrices_never_share_storage(make):
    st, _ = gs.from_board(make(), _device=False)
    sym = st.sym
    size = sym.nbnd.astype(np.int64) ** 2
    _check(sym.height, sym.parent, size, sym.upd_off, sym.upd_total)
    assert sym.upd_total <= size.sum()


def test_random_forests():
    rng = np.random.default_rng(3)
    for _ in range(20):
        n = int(rng.integers(1, 200))
        parent = np.full(n, -1, np.int64)
        for f in range(1, n):                      # a front's parent comes later in the order
            parent[f - 1] = int(rng.integers(f, n)) if rng.random() < 0.9 else -1
        height = np.zeros(n, np.int64)
        for f in range(n):
            if parent[f] >= 0:
                height[parent[f]] = max(height[parent[f]], height[f] + 1)
        size = rng.integers(0, 50, n).astype(np.int64)
        size[parent < 0] = 0                        # roots pass nothing up
        off, total = layout.update_slots(height, parent, size)
        _check(height, parent, size, off, total)
        assert total <= size.sum()
