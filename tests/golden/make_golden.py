"""Generate the golden fixtures in this folder by running GroundTruth's own FP64 solver.

Run in a container that has the reference checked out (it is read-only and never travels with the tests):

    python tests/golden/make_golden.py --reference /path/to/GroundTruth [--full]

The reference's solver module imports shapely at module level but uses it only to rasterise copper
(peec.build_grid), so a stub module is installed before the import and the rasterised grids come from
``groundtruth_gb300.synth`` (the same masks the GPU build solves).  For each board the script records:

* the board itself (masks, heights, pairs, branches, nets, frequencies)
* the reference's topology (strip lists, node ids, reference nodes, incidence ends)
* kernel quadrants, L_self, centre / sum values, sheet blocks
* the operator at the first frequency (R_strip, z_tail, D^-1, S as COO) and the products
  matvec(x), precond(x), Lp_matvec(I) on seeded vectors
* per net and frequency the solve at rtol = board.tol with GMRES(board.restart): unknown vector, its,
  Z_loop, magnetic moment, psi

``necked_pair.npz`` holds the same records for a plane pair with strips narrower than the pitch (an island on
a neck; the grids' wx / wy, ox / oy, rx / ry), plus the reference's strip widths, dL and M_near.
``faces_stack3_diag.npz`` / ``faces_stack3_sheet.npz``: three planes with screening on (the middle one split
into two face sheets, PlaneStack._faces), with either preconditioner, plus the sheets' layers, heights and twin
pairs and the face coupling Z12; ``necked_faces.npz`` the sheet-preconditioned one with narrow strips on the
split layer and the top one (the faces' shared corrections).
``necked_pair_scaled.npz`` / ``faces_stack3_sheet_scaled.npz``: those boards with seeded resistance factors on
every strip and branch (PlaneStack.set_resistance_scale): products and solves.
``necked_pair_fields.npz``: the reference's current-density maps of that board's net 0 (per cell and per
copper width, Solution.node_field; the real vectors at the dominant phase, the layers' current shares).
``small_pair_derived.npz`` holds the same for small_pair plus a what-if edit's branches on a derived stack
(PlaneStack.with_branches), including solves warm-started from the base's solutions.

``routed_pair.npz``: the same records for a plane pair rasterised from polygons by this build's restatement of
the reference's build_grid (raster.build_layer, sub-grid 4: exact widths, cell fills, measured node areas;
synth.routed_pair); ``routed_pair_fields.npz`` its current-density maps.
``known_answers.npz``: the reference's loop impedances and moments for the known-answer boards (the
microstrip over a 40 x 20 mm plane with and without slots or an edge cut, the parallel-plate lines 20 and 40 mm
long; ``synth.KNOWN_BOARDS``), solved to rtol 1e-10.

``--full`` additionally runs the 256 x 256 slotted plane pair (a few nets x frequencies, minutes per solve)
and stores only its scalar outputs (Z_loop, its, current norms).  ``--currents-only`` stores the reference's
full plane current maps (I_x, I_y) of three of its columns across the band (slotted_pair_currents.npz), which
the benchmark compares the GPU build's solution with.
"""
from __future__ import annotations

import argparse
import math
import sys
import time
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from groundtruth_gb300 import synth  # noqa: E402


def import_reference(root: str):
    sys.modules.setdefault("shapely", types.ModuleType("shapely"))
    sys.path.insert(0, str(Path(root) / "src"))
    from groundtruth.solver import kernel, peec  # noqa: E402
    return peec, kernel


def build_reference(peec, board: synth.Board):
    grids = [peec.Grid(0.0, 0.0, board.d * 1e3, board.nx, board.ny, l.node.copy(), l.xb.copy(), l.yb.copy(),
                       **{k: np.array(v, float) for k, v in (l.widths or {}).items()},
                       **{k: np.array(getattr(l, k)) for k in synth.CELL_KEYS if getattr(l, k) is not None})
             for l in board.layers]
    layers = [peec.PlaneLayer(l.name, l.z, g, l.thickness) for l, g in zip(board.layers, grids)]
    branches = [peec.Branch(b.a, b.b, (lambda f, b=b: b.z(f)), f"br{n}", b.kind, b.radius)
                for n, b in enumerate(board.branches)]
    pairs = [peec.PlanePair(p.upper, p.lower, p.c_per_area, p.tan_delta) for p in board.pairs]
    st = peec.PlaneStack(layers, branches, pairs, board.sigma, precond=board.precond, screen=board.screen)
    routes = []
    for net in board.nets:
        trace = [peec.TraceSegment(s[0:3].copy(), s[3:6].copy(), float(s[6]), float(s[7])) for s in net.segments]
        routes.append(peec.RouteExcitation(st, trace, net.driver, net.receiver, net.trace_t))
    return st, routes


def coo(M):
    M = M.tocoo()
    return np.stack([M.row, M.col]).astype(np.int64), M.data


def record(peec, board: synth.Board, solve: bool = True) -> dict:
    peec.gmres_restart = lambda n, r=board.restart: r
    peec.PlaneStack.solve.__defaults__ = (board.tol, 8, None)
    st, routes = build_reference(peec, board)
    out = {f"board_{k}": v for k, v in board.to_arrays().items()}
    out.update(xa=st.xa, ya=st.ya, nid=st.nid, keep=st.keep, a_nodes=st.a_nodes, b_nodes=st.b_nodes,
               full_label=st.full_label, cond_label=st.cond_label, Px=np.array(st.Px), Py=np.array(st.Py),
               Kq_x=st._kq["x"], Kq_y=st._kq["y"], L_self=np.float64(st.L_self), nb=np.int64(st.nb),
               ns=np.int64(st.ns), ncap=np.int64(st.ncap), nbr=np.int64(st.nbr), cap=st.cap)
    if getattr(st, "B_x", None) is not None:
        out.update(B_x=st.B_x, B_y=st.B_y)
    if len(getattr(st, "twin_parent", [])):          # split layers: face sheets
        out.update(n_sheets=np.int64(st.n_sheets), sheet_layer=st.sheet_layer, twin_parent=st.twin_parent,
                   tw_a=st.tw_a, tw_b=st.tw_b, sheet_z=st.sheet_z, sheet_t=st.sheet_t)
    if getattr(st, "dL", None) is not None:          # strips narrower than the pitch
        out.update(strip_width=st.strip_width, r_width=st.r_width, dL=st.dL)
        if st.M_near is not None:
            out["M_near_ij"], out["M_near"] = coo(st.M_near)
    f0 = float(board.freqs[0])
    op = st.operator(f0)
    out.update(op_f=np.float64(f0), op_R=op.R_strip, op_z=op.z_tail)
    if getattr(op, "Z12", None) is not None:
        out["op_Z12"] = op.Z12
    out["op_Dinv_ij"], out["op_Dinv"] = coo(op.Dinv)
    S = (st.ArT @ op.Dinv @ st.Ar)
    out["op_S_ij"], out["op_S"] = coo(S)
    rng = np.random.default_rng(123)
    n = st.nb + st.Ar.shape[1]
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    I = rng.standard_normal(st.ns) + 1j * rng.standard_normal(st.ns)
    host = peec._HostMath(st)
    out.update(prod_x=x, prod_matvec=host.matvec(op, x), prod_precond=host.precond(op, x), prod_I=I,
               prod_Lp=st.Lp_matvec(I))
    for k, r in enumerate(routes):
        out[f"psi{k}"] = r.psi
        out[f"Ltrace{k}"] = np.float64(r.L_trace)
        if not solve:
            continue
        for q, f in enumerate(board.freqs):
            t0 = time.perf_counter()
            sol = r.solve(float(f))
            out[f"Z{k}_{q}"] = np.complex128(sol.Z_loop)
            out[f"m{k}_{q}"] = sol.m
            out[f"its{k}_{q}"] = np.int64(sol.iterations)
            out[f"x{k}_{q}"] = sol.state_for(st)
            print(f"  {board.name} net {k} f {f:.4g}: its {sol.iterations} Z {sol.Z_loop:.6g} "
                  f"({time.perf_counter() - t0:.1f} s)", flush=True)
    return out


def record_derived(peec, board: synth.Board, seed: int) -> dict:
    """The same board plus a what-if edit's branches (synth.what_if_branches) on a derived stack
    (PlaneStack.with_branches: the base's factorisation with a Woodbury update): its operator's products on a
    seeded vector at the first frequency, and per net and frequency the cold solve and the solve warm-started
    from the base's solution (map_state)."""
    peec.gmres_restart = lambda n, r=board.restart: r
    peec.PlaneStack.solve.__defaults__ = (board.tol, 8, None)
    st, routes = build_reference(peec, board)
    extra = synth.what_if_branches(board, seed)
    branches = [peec.Branch(b.a, b.b, (lambda f, b=b: b.z(f)), f"x{n}", b.kind, b.radius) for n, b in enumerate(extra)]
    dst = st.with_branches(branches)
    assert dst._base is st, "the edit must make a derived stack"
    out = {f"board_{k}": v for k, v in board.to_arrays().items()}
    out["extra"] = np.array([[*b.a, *b.b, b.R, b.L, b.C, b.kind == "via", b.radius] for b in extra], float)
    out.update(nb=np.int64(dst.nb), nbr=np.int64(dst.nbr))
    f0 = float(board.freqs[0])
    op = dst.operator(f0)
    rng = np.random.default_rng(321)
    n = dst.nb + dst.Ar.shape[1]
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    host = peec._HostMath(dst)
    out.update(prod_x=x, prod_matvec=host.matvec(op, x), prod_precond=host.precond(op, x))
    for k, r in enumerate(routes):
        rd = r.on(dst)
        out[f"psi{k}"] = rd.psi
        for q, f in enumerate(board.freqs):
            base = r.solve(float(f))
            cold = rd.solve(float(f))
            warm = rd.solve(float(f), guess=[dst.map_state(base.state_for(st), st)])
            out[f"Z{k}_{q}"] = np.complex128(cold.Z_loop)
            out[f"x{k}_{q}"] = cold.state_for(dst)
            out[f"its{k}_{q}"] = np.int64(cold.iterations)
            out[f"Zwarm{k}_{q}"] = np.complex128(warm.Z_loop)
            out[f"itswarm{k}_{q}"] = np.int64(warm.iterations)
            print(f"  {board.name}+edit net {k} f {f:.4g}: its {cold.iterations} (warm {warm.iterations}) "
                  f"Z {cold.Z_loop:.6g}", flush=True)
    return out


def record_scaled(peec, board: synth.Board, seed: int) -> dict:
    """The board with seeded resistance factors on every strip (1.0-1.4) and branch (PlaneStack.
    set_resistance_scale): the operator's products at the first frequency and the solves."""
    rng = np.random.default_rng(seed)
    peec.gmres_restart = lambda n, r=board.restart: r
    peec.PlaneStack.solve.__defaults__ = (board.tol, 8, None)
    st, routes = build_reference(peec, board)
    rs, bs = rng.uniform(1.0, 1.4, st.ns), rng.uniform(1.0, 1.4, st.nbr)
    st.set_resistance_scale(rs, bs)
    out = {f"board_{k}": v for k, v in board.to_arrays().items()}
    out.update(r_scale=rs, branch_scale=bs)
    f0 = float(board.freqs[0])
    op = st.operator(f0)
    out.update(op_f=np.float64(f0), op_R=op.R_strip, op_z=op.z_tail)
    if getattr(op, "Z12", None) is not None:
        out["op_Z12"] = op.Z12
    rng2 = np.random.default_rng(123)
    n = st.nb + st.Ar.shape[1]
    x = rng2.standard_normal(n) + 1j * rng2.standard_normal(n)
    host = peec._HostMath(st)
    out.update(prod_x=x, prod_matvec=host.matvec(op, x), prod_precond=host.precond(op, x))
    for k, r in enumerate(routes):
        for q, f in enumerate(board.freqs):
            sol = r.solve(float(f))
            out[f"Z{k}_{q}"] = np.complex128(sol.Z_loop)
            out[f"x{k}_{q}"] = sol.state_for(st)
            print(f"  {board.name} scaled net {k} f {f:.4g}: its {sol.iterations} Z {sol.Z_loop:.6g}", flush=True)
    return out


def branch_functions(peec) -> dict:
    """The reference's via and track branch impedances at a few sizes and frequencies."""
    f = np.logspace(3, 10, 12)
    vias = [(1.6e-3, 0.3e-3, False), (0.2e-3, 0.2e-3, False), (1.0e-3, 0.8e-3, True), (0.0, 0.05e-3, False)]
    tracks = [(2e-3, 0.15e-3, 35e-6), (0.5e-3, 0.4e-3, 18e-6), (5e-3, 1e-3, 70e-6)]
    out = {"bf_f": f, "bf_via_args": np.array(vias, float), "bf_track_args": np.array(tracks, float)}
    out["bf_via"] = np.array([[peec.via_impedance(l, dr, filled=fl)(x) for x in f] for l, dr, fl in vias])
    out["bf_track"] = np.array([[peec.track_impedance(l, w, t)(x) for x in f] for l, w, t in tracks])
    return out


def record_fields(peec, board: synth.Board) -> dict:
    """The reference's current-density maps (Solution.node_field, per cell and per copper width) of net 0 at
    the board's second frequency, every layer."""
    peec.gmres_restart = lambda n, r=board.restart: r
    peec.PlaneStack.solve.__defaults__ = (board.tol, 8, None)
    st, routes = build_reference(peec, board)
    f = float(board.freqs[1])
    sol = routes[0].solve(f)
    out = {f"board_{k}": v for k, v in board.to_arrays().items()}
    out.update(f=np.float64(f), x=sol.state_for(st))
    for k in range(st.N):
        for copper in (False, True):
            kx, ky = sol.node_field(k, board.d * 1e3, copper=copper)
            out[f"kx{k}_{int(copper)}"], out[f"ky{k}_{int(copper)}"] = kx, ky
            vx, vy = sol.sheet_vectors(k, board.d * 1e3, copper=copper)
            out[f"vx{k}_{int(copper)}"], out[f"vy{k}_{int(copper)}"] = vx, vy
    out.update(phase=np.float64(sol.dominant_phase()), share=sol.layer_share(),
               share_masked=sol.layer_share([(np.ones_like(sol.I_x[k].real, bool), np.zeros_like(sol.I_y[k].real, bool))
                                             for k in range(st.N)]))
    return out


def kernel_functions(kernel) -> dict:
    """Point values of the reference's Green's-function helpers."""
    rng = np.random.default_rng(7)
    L, ax, rho = 1e-3 * rng.uniform(0.1, 2, 40), 1e-3 * rng.uniform(-5, 5, 40), 1e-3 * rng.uniform(1e-3, 5, 40)
    tape_args = np.array([[1e-3, 1e-3, 1e-3, 0.0, 0.0, 0.0], [0.5e-3, 0.5e-3, 0.5e-3, 0.5e-3, 0.5e-3, 0.2e-3],
                          [0.25e-3, 0.25e-3, 0.25e-3, 0.0, 0.75e-3, 1.0e-3], [1e-3, 0.3e-3, 0.7e-3, 2e-3, -0.4e-3, 0.0],
                          [0.4e-3, 0.4e-3, 0.4e-3, 1.2e-3, 1.6e-3, 1.07e-3]])
    f = np.logspace(3, 10, 30)
    return {"fm_args": np.stack([L, ax, rho]), "fm": kernel.filament_mutual(L, ax, rho),
            "tape_args": tape_args, "tape": np.array([kernel.tape_mutual(*a) for a in tape_args]),
            "ssn_w": np.array([0.1e-3, 0.25e-3, 1e-3]), "ssn": kernel.strip_self_numeric(1e-3, np.array([0.1e-3, 0.25e-3, 1e-3])),
            "sk_f": f, "skin35": kernel.skin_thickness(35e-6, f, 5.8e7), "slab18": kernel.slab_impedance(18e-6, f, 5.8e7),
            "slab35": kernel.slab_impedance(35e-6, f, 5.8e7),
            "strip_kernel_6x5": kernel.strip_kernel(6, 5, 0.5e-3, 0.3e-3)}


KNOWN_TOL = 1e-10


def record_known(peec) -> dict:
    """Per known-answer board and frequency the reference's Z_loop, moment and iterations at rtol KNOWN_TOL."""
    out = {}
    for name, make in synth.KNOWN_BOARDS.items():
        board = make()
        peec.gmres_restart = lambda n, r=board.restart: r
        peec.PlaneStack.solve.__defaults__ = (KNOWN_TOL, 8, None)
        st, routes = build_reference(peec, board)
        out[f"{name}_freqs"] = np.asarray(board.freqs, float)
        for q, f in enumerate(board.freqs):
            t0 = time.perf_counter()
            sol = routes[0].solve(float(f))
            out[f"{name}_Z{q}"] = np.complex128(sol.Z_loop)
            out[f"{name}_m{q}"] = np.asarray(sol.m)
            out[f"{name}_its{q}"] = np.int64(sol.iterations)
            print(f"  {name} f {f:.4g}: its {sol.iterations} Z {sol.Z_loop:.10g} ({time.perf_counter() - t0:.1f} s)",
                  flush=True)
    return out


# the full-size columns whose plane currents are stored: (net, frequency index) of the slotted pair's 8 nets x
# 32 frequencies, spanning the band (1 MHz, 28.3 MHz, 1 GHz)
CURRENT_COLUMNS = ((0, 0), (1, 15), (0, 31))


def record_currents(peec, board: synth.Board) -> dict:
    """The reference's own plane currents I_x, I_y (sheets x strips, rounded to complex64, far below the 1e-6
    the GPU build is held to) and Z_loop for CURRENT_COLUMNS of the full-size slotted pair, solved to board.tol
    with GMRES(board.restart)."""
    st, routes = build_reference(peec, board)
    peec.gmres_restart = lambda n, r=board.restart: r
    peec.PlaneStack.solve.__defaults__ = (board.tol, 8, None)
    out = {"cols": np.array(CURRENT_COLUMNS, np.int64), "freqs": np.asarray(board.freqs)}
    for n, (k, q) in enumerate(CURRENT_COLUMNS):
        t0 = time.perf_counter()
        sol = routes[k].solve(float(board.freqs[q]))
        out[f"Ix{n}"] = np.asarray(sol.I_x).astype(np.complex64)
        out[f"Iy{n}"] = np.asarray(sol.I_y).astype(np.complex64)
        out[f"Z{n}"] = np.complex128(sol.Z_loop)
        out[f"its{n}"] = np.int64(sol.iterations)
        print(f"  slotted_pair net {k} f {board.freqs[q]:.4g}: its {sol.iterations} Z {sol.Z_loop:.10g} "
              f"({time.perf_counter() - t0:.1f} s)", flush=True)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    ap.add_argument("--full", action="store_true")
    ap.add_argument("--derived-only", action="store_true", help="only the derived-stack fixture")
    ap.add_argument("--narrow-only", action="store_true", help="only the narrow-strip board's fixture")
    ap.add_argument("--faces-only", action="store_true", help="only the face-sheet boards' fixtures")
    ap.add_argument("--known-only", action="store_true", help="only the known-answer boards' scalars")
    ap.add_argument("--routed-only", action="store_true", help="only the board rasterised from polygons")
    ap.add_argument("--fields-only", action="store_true", help="only the current-density maps")
    ap.add_argument("--currents-only", action="store_true",
                    help="only the full-size slotted pair's plane currents (slotted_pair_currents.npz)")
    args = ap.parse_args()
    peec, kernel = import_reference(args.reference)
    if args.currents_only:
        np.savez_compressed(HERE / "slotted_pair_currents.npz", **record_currents(peec, synth.slotted_pair()))
        return
    if args.fields_only:
        np.savez_compressed(HERE / "necked_pair_fields.npz", **record_fields(peec, synth.necked_pair()))
        np.savez_compressed(HERE / "routed_pair_fields.npz", **record_fields(peec, synth.routed_pair()))
        return
    print("routed_pair", flush=True)
    np.savez_compressed(HERE / "routed_pair.npz", **record(peec, synth.routed_pair()))
    np.savez_compressed(HERE / "routed_pair_fields.npz", **record_fields(peec, synth.routed_pair()))
    if args.routed_only:
        return
    print("known_answers", flush=True)
    np.savez_compressed(HERE / "known_answers.npz", **record_known(peec))
    if args.known_only:
        return
    for pc in ("diag", "sheet"):
        print(f"faces_stack3_{pc}", flush=True)
        np.savez_compressed(HERE / f"faces_stack3_{pc}.npz", **record(peec, synth.faces_stack3(pc)))
    print("necked_faces", flush=True)
    np.savez_compressed(HERE / "necked_faces.npz", **record(peec, synth.necked_faces()))
    print("necked_pair_fields", flush=True)
    np.savez_compressed(HERE / "necked_pair_fields.npz", **record_fields(peec, synth.necked_pair()))
    for name in ("necked_pair", "faces_stack3_sheet"):
        board = synth.WORKLOADS[name]() if name != "faces_stack3_sheet" else synth.faces_stack3("sheet")
        print(f"{name}_scaled", flush=True)
        np.savez_compressed(HERE / f"{name}_scaled.npz", **record_scaled(peec, board, seed=31))
    if args.faces_only:
        return
    print("necked_pair", flush=True)
    np.savez_compressed(HERE / "necked_pair.npz", **record(peec, synth.necked_pair()))
    if args.narrow_only:
        return
    print("small_pair_derived", flush=True)
    np.savez_compressed(HERE / "small_pair_derived.npz", **record_derived(peec, synth.small_pair(), seed=11))
    if args.derived_only:
        return
    np.savez_compressed(HERE / "kernel_functions.npz", **kernel_functions(kernel), **branch_functions(peec))
    for name in ("small_pair", "small_stack3", "plain_plane"):
        board = synth.WORKLOADS[name]()
        print(name, flush=True)
        np.savez_compressed(HERE / f"{name}.npz", **record(peec, board))
    if args.full:
        board = synth.slotted_pair()
        sub = synth.slotted_pair()
        sub.nets = sub.nets[:2]
        sub.freqs = board.freqs[[0, 15, 31]]
        st, routes = build_reference(peec, sub)
        peec.gmres_restart = lambda n, r=sub.restart: r
        peec.PlaneStack.solve.__defaults__ = (sub.tol, 8, None)
        out = {"freqs": sub.freqs, "Px": np.array(st.Px), "Kq_x_sum": st._kq["x"].sum(axis=(0, 1)),
               "nb": np.int64(st.nb), "keep_count": np.int64(st.keep.sum())}
        for k, r in enumerate(routes):
            out[f"psi{k}_norm"] = np.float64(np.linalg.norm(r.psi))
            for q, f in enumerate(sub.freqs):
                t0 = time.perf_counter()
                sol = r.solve(float(f))
                out[f"Z{k}_{q}"] = np.complex128(sol.Z_loop)
                out[f"its{k}_{q}"] = np.int64(sol.iterations)
                out[f"Ixnorm{k}_{q}"] = np.linalg.norm(sol.I_x.reshape(2, -1), axis=1)
                out[f"Iynorm{k}_{q}"] = np.linalg.norm(sol.I_y.reshape(2, -1), axis=1)
                print(f"  slotted_pair net {k} f {f:.4g}: its {sol.iterations} Z {sol.Z_loop:.8g} "
                      f"({time.perf_counter() - t0:.1f} s)", flush=True)
        np.savez_compressed(HERE / "slotted_pair_scalars.npz", **out)


if __name__ == "__main__":
    main()
