"""The Python mirror's error behaviour, as the reference's (peec.py:124-127, 1559-1593, 2199-2216, 2713-2760):
SolverError for unsolvable models and bad injections, ValueError for malformed arguments.  Host side only."""
import numpy as np
import pytest

from groundtruth_gb300 import stack as gs, synth


def host(board):
    return gs.from_board(board, _device=False)


def test_no_layers_and_bad_preconditioner():
    with pytest.raises(gs.SolverError):
        gs.PlaneStack([], _device=False)
    b = synth.small_pair()
    st, _ = host(b)
    with pytest.raises(ValueError):
        gs.PlaneStack(st.layers, precond="ilu", _device=False)


def test_layers_must_share_one_grid():
    b = synth.small_pair()
    st, _ = host(b)
    g = st.layers[1].grid
    other = gs.Grid(0.0, 0.0, g.d, g.nx - 1, g.ny, g.node[:-1], g.xb[:-1], g.yb[:-1])
    with pytest.raises(gs.SolverError):
        gs.PlaneStack([st.layers[0], gs.PlaneLayer("X", -1e-3, other)], _device=False)


def test_injections_must_be_on_copper_and_balance():
    b = synth.small_pair()
    st, routes = host(b)
    trace = routes[0].trace
    hole = tuple(int(v) for v in np.argwhere(~st.node[0])[0])       # a node of the slot
    with pytest.raises(gs.SolverError, match="not on plane copper"):
        gs.RouteExcitation(st, trace, (0, *hole), b.nets[0].receiver)
    with pytest.raises(gs.SolverError, match="not on plane copper"):
        gs.RouteExcitation(st, trace, (0, st.nx + 5, 0), b.nets[0].receiver)      # off the grid
    with pytest.raises(gs.SolverError, match="no current"):
        gs.RouteExcitation(st, trace)
    with pytest.raises(gs.SolverError, match="balance"):
        gs.RouteExcitation(st, trace, injections=[(b.nets[0].driver, 1.0)])


def test_driver_and_receiver_on_separate_copper():
    b = synth.microstrip(full_cut=True)
    with pytest.raises(gs.SolverError, match="not connected"):
        host(b)


def test_resistance_factors_must_match_the_unknowns():
    st, _ = host(synth.small_pair())
    with pytest.raises(ValueError):
        st.set_resistance_scale(np.ones(st.ns - 1))
    with pytest.raises(ValueError):
        st.set_resistance_scale(None, np.ones(st.nbr + 1))


def test_branches_off_copper_are_dropped():
    b = synth.small_pair()
    st, _ = host(b)
    hole = tuple(int(v) for v in np.argwhere(~st.node[0])[0])
    br = gs.Branch((0, *hole), (1, *hole), lambda f: 1.0 + 0j)
    assert st.with_branches([br]) is st
    new = gs.PlaneStack(st.layers, st.branches + [br], st.pairs, precond="sheet", screen=False, _device=False)
    assert new.nbr == st.nbr


def test_plane_problem_builds_the_stack_and_route():
    """PlaneProblem (peec.py:2829-2837): one plane at z = 0 under a trace, (i, j) nodes taken as layer 0."""
    b = synth.microstrip()
    l = b.layers[0]
    g = gs.Grid(0.0, 0.0, b.d * 1e3, b.nx, b.ny, l.node, l.xb, l.yb)
    net = b.nets[0]
    trace = [gs.TraceSegment(s[0:3], s[3:6], float(s[6])) for s in net.segments]
    pp = gs.PlaneProblem(g, trace, net.driver[1:], net.receiver[1:], _device=False)
    st, routes = host(b)
    assert pp.stack.nb == st.nb and pp.injections == routes[0].injections
    assert np.allclose(pp.psi, routes[0].psi)


def test_face_z_and_surface_impedance():
    """PlaneStack.face_z (peec.py:1935-1939): a one-sheet layer's face towards a height is its centre moved half
    its copper that way; surface_impedance (2144-2148) is the one-face slab's."""
    from groundtruth_gb300 import greens
    st, _ = host(synth.small_pair())
    for k in range(st.n_sheets):
        up, down = st.face_z(k, 1.0), st.face_z(k, -1.0)
        assert up - down == pytest.approx(st.sheet_t[k]) and 0.5 * (up + down) == pytest.approx(st.sheet_z[k])
    assert st.surface_impedance(1e8, 35e-6) == complex(greens.slab_impedance(35e-6, 1e8, st.sigma))
