"""The what-if server (groundtruth_gb300.serve): requests that arrive together are answered from one batched
device solve per resident geometry, and each request's answers are the same as when it is served alone and as
the unbatched what-if service gives them, within the tolerance the columns are solved to.  Needs a GPU."""
import numpy as np
import pytest

from groundtruth_gb300 import serve, stack as gs, synth, whatif

pytestmark = pytest.mark.gpu
N, NETS, FREQS = 48, 4, 4


def _board(slot=True):
    return synth.what_if_base(n=N, n_nets=NETS, n_freq=FREQS, slot=slot, n_decap=3)


@pytest.fixture(scope="module")
def server():
    geos = {}
    for name, slot in (("base", True), ("toggled", False)):
        board = _board(slot)
        st, routes = gs.from_board(board)
        wi = whatif.WhatIf(st, routes, board.freqs, tol=1e-8, max_cols=256, reorth=0.0)
        wi.baseline()
        geos[name] = wi
    srv = serve.Server(geos, budget_bytes=40e9)
    yield srv, geos, _board()
    srv.close()


def _requests(board, geos):
    st = geos["base"].stack
    freqs = [float(f) for f in board.freqs]
    out = []
    for r in range(6):
        extra = synth.what_if_branches(board, seed=300 + r, n_via=1 + r % 3, n_part=0)
        br = [gs.Branch(b.a, b.b, b.z, f"edit{r}_{n}", b.kind, b.radius) for n, b in enumerate(extra)]
        out.append(serve.Request(nets=[r % NETS, (r + 1) % NETS], freqs=freqs[r % 2::2], branches=br,
                                 remove=[r % st.nbr] if r % 3 == 2 else []))
    out.append(serve.Request(nets=[0, 2], freqs=freqs[1:3], geometry="toggled"))
    return out


def _same(a, b, rel=1e-9):
    assert set(a.solutions) == set(b.solutions)
    for c in a.solutions:
        za, zb = a.solutions[c].Z_loop, b.solutions[c].Z_loop
        assert abs(za - zb) <= rel * abs(zb), (c, za, zb)


def test_each_request_is_the_same_alone_and_in_the_mix(server):
    srv, geos, board = server
    reqs = _requests(board, geos)
    alone = [srv.submit(r).result(timeout=600) for r in reqs]
    futs = [srv.submit(r) for r in reqs]          # submitted together: served in one or two batches
    mixed = [f.result(timeout=600) for f in futs]
    assert max(m.batch_requests for m in mixed) > 1
    for a, m in zip(alone, mixed):
        _same(a.result, m.result)
        assert all(c.residual <= 1e-8 for c in m.result.solutions.values())
    # and the unbatched service agrees
    for r, m in zip(reqs[:3], mixed[:3]):
        ref = geos["base"].evaluate(r.branches, r.nets, r.freqs, remove=r.remove)
        _same(m.result, ref)


def test_a_slot_toggle_solves_on_its_own_resident_geometry(server):
    srv, geos, board = server
    f = float(board.freqs[0])
    ans = srv.submit(serve.Request(nets=[1], freqs=[f], geometry="toggled")).result(timeout=600)
    ref = geos["toggled"].base[(1, f)]
    got = ans.result.solutions[(1, f)]
    assert abs(got.Z_loop - ref.Z_loop) <= 1e-6 * abs(ref.Z_loop)
