"""The board dispatcher's failure handling (GroundTruth's compute server: one job per worker process under a
watchdog, remote/worker.py:1-30), on the CPU: a worker killed in the middle of a batch has its job finished by its
replacement, a job that hangs is cut off at its time limit, a job that raises is reported and not retried, and the
other jobs of the batch come back unaffected.  The serving test runs the oracle's solve in the workers, so the jobs
are real solves; the product's job function (dispatch.solve_board) is the same call on the GPU library."""
import os
import time
from pathlib import Path

import numpy as np
import pytest

from groundtruth_gb300 import dispatch, synth


def _job(p):
    kind = p["kind"]
    if kind == "square":
        return p["x"] ** 2
    if kind == "die_once":                  # the first worker to get it dies; the next one finishes it
        marker = Path(p["marker"])
        if not marker.exists():
            marker.write_text("died")
            os._exit(3)
        return "second try"
    if kind == "die":
        os._exit(4)
    if kind == "hang":
        time.sleep(120)
    if kind == "raise":
        from groundtruth_gb300.stack import SolverError
        raise SolverError("GMRES did not converge at 1 MHz")
    if kind == "device":
        return os.environ.get("CUDA_VISIBLE_DEVICES"), os.getpid()
    raise ValueError(kind)


def _oracle_job(p):
    """One (net, frequency) of a board through the oracle; with a marker, the first worker to get it dies after
    building the stack, in the middle of the job."""
    from test_oracle_golden import oracle_routes, oracle_stack
    board = synth.Board.from_arrays(p["board"])
    route = oracle_routes(oracle_stack(board), board)[p["net"]]
    if p.get("marker") and not Path(p["marker"]).exists():
        Path(p["marker"]).write_text("died")
        os._exit(5)
    out = route.solve(float(board.freqs[p["f"]]), tol=board.tol)
    return complex(out["Z_loop"]), np.asarray(out["m"])


def test_results_come_back_in_order_from_every_worker():
    with dispatch.Dispatcher(_job, workers=2) as d:
        out = d.map([{"kind": "square", "x": x} for x in range(12)])
        assert [o.value for o in out] == [x * x for x in range(12)]
        assert all(o.ok and o.attempts == 1 and o.error is None for o in out)
        assert {o.worker for o in out} == {0, 1}
        assert d.replaced == 0
        assert d.map([]) == []


def test_a_worker_killed_mid_batch_is_replaced_and_its_job_redone(tmp_path):
    jobs = [{"kind": "square", "x": x} for x in range(6)]
    jobs[2] = {"kind": "die_once", "marker": str(tmp_path / "m")}
    with dispatch.Dispatcher(_job, workers=2) as d:
        out = d.map(jobs)
        assert out[2].ok and out[2].value == "second try" and out[2].attempts == 2
        assert [o.value for k, o in enumerate(out) if k != 2] == [x * x for x in range(6) if x != 2]
        assert d.replaced == 1
        assert all(p.is_alive() for p in d.procs)
        assert d.map([{"kind": "square", "x": 7}])[0].value == 49      # the pool still serves


def test_a_job_that_always_kills_its_worker_is_reported_lost():
    with dispatch.Dispatcher(_job, workers=2, attempts=3) as d:
        out = d.map([{"kind": "die"}, {"kind": "square", "x": 3}])
        assert not out[0].ok and out[0].error.startswith("WorkerLost: worker exited with code 4")
        assert out[0].attempts == 3 and d.replaced == 3
        assert out[1].ok and out[1].value == 9


def test_a_hung_job_is_cut_off_at_its_time_limit():
    with dispatch.Dispatcher(_job, workers=1, timeout=1.0, attempts=2) as d:
        t0 = time.monotonic()
        out = d.map([{"kind": "hang"}, {"kind": "square", "x": 5}])
        assert time.monotonic() - t0 < 60
        assert not out[0].ok and out[0].error.startswith("WorkerLost: timed out after 1 s")
        assert out[0].attempts == 2
        assert out[1].ok and out[1].value == 25


def test_a_job_that_raises_is_reported_and_not_retried():
    with dispatch.Dispatcher(_job, workers=1) as d:
        out = d.map([{"kind": "raise"}, {"kind": "square", "x": 2}])
        assert not out[0].ok and out[0].attempts == 1
        assert out[0].error == "SolverError: GMRES did not converge at 1 MHz"
        assert out[1].value == 4 and d.replaced == 0


def test_each_worker_owns_its_device():
    with dispatch.Dispatcher(_job, workers=2, devices=[3, 5]) as d:
        seen = {}
        for o in d.map([{"kind": "device"}] * 8):
            seen.setdefault(o.worker, set()).add(o.value[0])
        assert all(seen[w] == {str(dev)} for w, dev in zip((0, 1), (3, 5)) if w in seen)
        procs = list(d.procs)
    assert not any(p.is_alive() for p in procs)             # close() stopped them


def test_bad_arguments():
    with pytest.raises(ValueError):
        dispatch.Dispatcher(_job, workers=0)
    with pytest.raises(ValueError):
        dispatch.Dispatcher(_job, workers=2, devices=[0])
    with pytest.raises(ValueError):
        dispatch.Dispatcher(_job, attempts=0)


def test_serving_solves_survive_a_worker_killed_mid_batch(tmp_path):
    """Four solves of a board served by two workers, one of which dies in the middle of its solve: every loop
    impedance and moment equals the same solve run here."""
    from test_oracle_golden import oracle_routes, oracle_stack
    board = synth.small_pair()
    arrays = board.to_arrays()
    jobs = [{"board": arrays, "net": k, "f": i} for k in range(len(board.nets)) for i in (0, 2)]
    jobs[1]["marker"] = str(tmp_path / "killed")
    with dispatch.Dispatcher(_oracle_job, workers=2) as d:
        out = d.map(jobs)
    assert (tmp_path / "killed").exists()
    assert all(o.ok for o in out) and out[1].attempts == 2
    routes = oracle_routes(oracle_stack(board), board)
    for j, o in zip(jobs, out):
        ref = routes[j["net"]].solve(float(board.freqs[j["f"]]), tol=board.tol)
        assert o.value[0] == pytest.approx(complex(ref["Z_loop"]), rel=1e-12)
        assert np.allclose(o.value[1], ref["m"], rtol=1e-12, atol=0)


def test_solve_board_reads_the_board_and_gathers_every_net_and_frequency(monkeypatch):
    """dispatch.solve_board's host side, in this process: the board comes back from its arrays, every net is solved
    at every frequency in one batch, and the answers are gathered per (net, frequency).  The device solve is
    replaced here by the oracle's."""
    from groundtruth_gb300 import stack as gs
    from test_oracle_golden import oracle_routes, oracle_stack
    board = synth.small_pair()
    host = gs.from_board
    monkeypatch.setattr(gs, "from_board", lambda b: host(b, _device=False))
    seen = {}

    def oracle_many(routes, freqs, tol, restart):
        seen.update(n=len(routes), freqs=list(freqs), tol=tol, restart=restart)
        ref = oracle_routes(oracle_stack(board), board)
        out = []
        for r in ref:
            row = []
            for f in freqs:
                o = r.solve(float(f), tol=tol)
                row.append(gs.Solution(float(f), o["I_x"], o["I_y"], o["V"], o["I_branch"], complex(o["Z_loop"]),
                                       np.asarray(o["m"]), int(o["its"])))
            out.append(row)
        return out
    monkeypatch.setattr(gs, "solve_many", oracle_many)
    res = dispatch.solve_board(board.to_arrays())
    nn, nf = len(board.nets), len(board.freqs)
    assert seen == dict(n=nn, freqs=list(board.freqs), tol=board.tol, restart=board.restart)
    assert res["Z_loop"].shape == (nn, nf) and res["m"].shape == (nn, nf, 3)
    assert res["iterations"].shape == (nn, nf) and res["residual"].shape == (nn, nf)
    assert np.array_equal(res["freqs"], board.freqs)
    ref = oracle_routes(oracle_stack(board), board)[1].solve(float(board.freqs[2]), tol=board.tol)
    assert res["Z_loop"][1, 2] == complex(ref["Z_loop"])
