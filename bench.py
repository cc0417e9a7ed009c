#!/usr/bin/env python
"""Benchmark of the GB300 PEEC plane-current solve.

Workload (the reference's precision + batching configuration): a 4-layer Sig/GND/PWR/Sig board, 256 x 256
cells at 0.25 mm, a seeded 1 mm slot across 60 % of the GND plane, 8 random-walk nets crossing it, 32
log-spaced frequencies 1 MHz - 1 GHz: 256 solves per step, each to a relative FP64 residual of 1e-10 (the
tolerance the FP64 oracle solves to).  A step solves all 256 columns in one batched device run.

    python bench.py [--gpus N --steps K --warmup W]          this build (one JSON line on rank 0)
    python bench.py --impl reference [...]                    the reference algorithm on the host CPU

value: solves/s with the right-hand sides resident in HBM and each frequency's factorised preconditioner
resident (factorisation time reported beside it); e2e: solves/s through the C ABI from host buffers,
every step factorising all 32 frequencies and copying the right-hand sides in and the solutions out.
Multi-GPU runs are replicas (every rank solves its own copy of the batch; no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "PEEC solves/s @<=1e-6 rel err vs FP64 oracle"
WORKLOAD = "slotted_pair 4-layer 256x256 @0.25mm, slot, 8 nets x 32 freqs (1 MHz-1 GHz)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--restart", type=int, default=50)
    ap.add_argument("--inner-tol", type=float, default=1e-5)
    ap.add_argument("--cpu-cols", type=int, default=16,
                    help="columns of the CPU baseline, solved whole side by side on the host cores")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 GPU comparator")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end (host buffers) leg")
    ap.add_argument("--e2e-chunks", type=int, default=1,
                    help="e2e: frequency groups factorised while earlier groups solve (native.solve_sweep); 1 "
                         "(default): factorise every frequency, then solve all columns in one batch — measured "
                         "faster here (4 groups: 8.16 s a step against 6.9 s: four 64-column solves pay the "
                         "sweeps' latency-bound top levels and the per-step host work four times)")
    ap.add_argument("--reorth", type=float, default=0.0,
                    help="DGKS re-orthogonalisation ratio (0.7: the reference rule; 0: none, the FP64 refinement guards the answer)")
    ap.add_argument("--max-its", type=int, default=4000)
    ap.add_argument("--outer-k", type=int, default=8, help="FP64 outer GCR directions kept (1: plain refinement)")
    ap.add_argument("--nets", type=int, default=0, help="use only the first N nets (0: all)")
    ap.add_argument("--freqs", type=int, default=0, help="use only every k-th frequency (0: all)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "mixed16"],
                    help="inner GMRES: FP32 with an FP32 (mixed) or FP16 (mixed16) Krylov basis")
    ap.add_argument("--borrow", action="store_true",
                    help="precondition every other frequency with its neighbour's factorisation (half the LDL^T)")
    ap.add_argument("--levels", action="store_true",
                    help="also time each elimination level of the triangular solves (key 'solve_levels')")
    ap.add_argument("--boards", type=int, default=64, help="uneven: boards in the batch")
    ap.add_argument("--concurrency", type=int, default=8, help="uneven: boards in flight at once")
    ap.add_argument("--no-alone", action="store_true", help="uneven: skip the one-board-at-a-time pass")
    ap.add_argument("--budget-gb", type=float, default=120.0, help="serve: device-memory budget (GB)")
    ap.add_argument("--side", type=int, default=1024, help="largest: raster side (nodes per axis)")
    ap.add_argument("--largest-nets", type=int, default=16, help="largest: nets solved (of 32)")
    ap.add_argument("--largest-freqs", type=int, default=1, help="largest: frequencies solved (of 64)")
    ap.add_argument("--workload", default="slotted_pair", choices=["slotted_pair", "what_if", "uneven", "serve", "largest"],
                    help="what_if: latency of interactive edits (added vias / decoupling parts) on a solved "
                         "512 x 512 board, warm-started derived stacks (a line of its own, not the headline)")
    ap.add_argument("--requests", type=int, default=24, help="what_if: timed edits")
    ap.add_argument("--rate", type=float, default=200.0, help="what_if: Poisson arrival rate (edits/s) of the queue")
    ap.add_argument("--max-cols", type=int, default=32, help="what_if: columns per device batch")
    ap.add_argument("--border-tol", type=float, default=0.1,
                    help="what_if: tolerance of the border solves relative to --tol's (bordered)")
    ap.add_argument("--what-if-method", default="bordered", choices=["bordered", "derived"],
                    help="what_if: compose from base solves (bordered) or solve every column on the derived stack")
    return ap.parse_args()


# DRAM bytes (read + write) over algorithmic bytes of one launch, from ncu captures of the Gram-Schmidt
# kernels on 32 columns of this workload (a launch with 31 basis vectors): no re-reads.  The roofline's
# traffic scales the live per-launch algorithmic bytes by it.
TRAFFIC_RATIO = {"gs_dots_f32": 1.002, "gs_update_f32": 0.999}
MULTI_KERNEL_REGIONS = {"fwdbwd_f32", "fwdbwd_f64", "fwd_f32", "bwd_f32", "fwd_f64", "bwd_f64", "gcr", "gmres_small",
                        "norms"}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------------------------------------ clocks
class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = [l.split(",") for l in Path(self.f.name).read_text().splitlines() if l.strip()]
        sm = [float(r[1]) for r in rows if len(r) > 8 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 8 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            if len(r) > 8:
                for k, n in enumerate(names):
                    if "Active" in r[5 + k] and "Not" not in r[5 + k]:
                        reasons.add(n)
        os.unlink(self.f.name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------------ CPU side
THREAD_VARS = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS", "BLIS_NUM_THREADS")


def cpu_columns(n: int, n_nets: int, n_freqs: int) -> list:
    """n (net, frequency index) columns of the workload spread over the band: frequency indices evenly from the
    first to the last, the nets in turn."""
    if n <= 1:
        return [(0, n_freqs // 2)]
    return [(i % n_nets, int(round(i * (n_freqs - 1) / (n - 1)))) for i in range(n)]


def _oracle_stack(board):
    from oracle import peec_oracle as po
    layers = [po.OLayer(l.z, l.thickness, l.node, l.xb, l.yb) for l in board.layers]
    return po.OracleStack(layers, board.d, [], [po.OPair(p.upper, p.lower, p.c_per_area, p.tan_delta)
                                                for p in board.pairs], board.sigma, board.precond)


def _cpu_worker(cols: list, ready, start, out) -> None:
    """A CPU-baseline worker process (single-threaded numerics): builds the oracle stack and factorises each of
    its columns' operators (untimed), reports ready, waits for the common start, then solves each column whole
    to the board's tolerance (the reference's restarted GMRES with its Schur preconditioner) and reports the
    wall-clock span of every solve."""
    try:
        from groundtruth_gb300 import synth
        from oracle import peec_oracle as po
        po.FFT_WORKERS = 1
        board = synth.slotted_pair()
        st = _oracle_stack(board)
        routes, jobs, t_fact = {}, [], 0.0
        for k, q in cols:
            if k not in routes:
                n0 = board.nets[k]
                routes[k] = po.OracleRoute(st, [po.OSegment(s[0:3].copy(), s[3:6].copy(), float(s[6]), float(s[7]))
                                                for s in n0.segments], n0.driver, n0.receiver, n0.trace_t)
            f = float(board.freqs[q])
            t0 = time.perf_counter()
            op = st.operator(f)
            t_fact += time.perf_counter() - t0
            jobs.append((k, q, op, np.concatenate([routes[k].rhs_top(f), routes[k].J()[st.keep].astype(complex)])))
        ready.put(("ready", t_fact))
        start.wait()
        done = []
        for k, q, op, rhs in jobs:
            t0 = time.time()
            x, its, ok = po.gmres(lambda v, op=op: st.matvec(op, st.precond(op, v)), rhs, board.tol, max_cycles=8,
                                  restart=board.restart, extra_cycles=po.GMRES_EXTRA_CYCLES)
            done.append((k, q, t0, time.time(), int(its), bool(ok)))
        out.put(("done", done))
    except Exception as e:                      # reported to the parent, which raises it
        ready.put(("error", repr(e)))
        out.put(("error", repr(e)))


def cpu_pool(columns: list, workers: int, freqs, timeout: float = 3600.0) -> dict:
    """Whole solves of `columns` by the reference algorithm (the oracle port: FP64, scipy FFTs, SuperLU,
    restarted GMRES to the board's tolerance) on `workers` single-threaded processes of this host, the columns
    dealt out in turn.  Operators are factorised before the timed region (as the GPU's `value` has them
    resident); the timed region runs from the common start to the last solve's end."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    ready, out, start = ctx.Queue(), ctx.Queue(), ctx.Event()
    shares = [columns[w::workers] for w in range(workers)]
    shares = [c for c in shares if c]
    saved = {k: os.environ.get(k) for k in THREAD_VARS}
    for k in THREAD_VARS:
        os.environ[k] = "1"
    try:
        procs = [ctx.Process(target=_cpu_worker, args=(c, ready, start, out), daemon=True) for c in shares]
        for p in procs:
            p.start()
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    fact = []
    for _ in procs:
        kind, val = ready.get(timeout=timeout)
        if kind != "ready":
            raise RuntimeError(f"CPU baseline worker failed: {val}")
        fact.append(val)
    t_start = time.time()
    start.set()
    solves = []
    for _ in procs:
        kind, val = out.get(timeout=timeout)
        if kind != "done":
            raise RuntimeError(f"CPU baseline worker failed: {val}")
        solves += val
    for p in procs:
        p.join(timeout=60)
    wall = max(s[3] for s in solves) - t_start
    per = [s[3] - s[2] for s in solves]
    return {"value": len(solves) / wall, "unit": "solves/s", "cores": len(procs), "kind": "port",
            "sample": (f"{len(solves)} whole solves (rtol 1e-10, GMRES(50) + Schur preconditioner, FP64; columns "
                       f"(net, f) {[(int(k), round(float(freqs[q]) / 1e6, 3)) for k, q, *_ in solves]} MHz) by "
                       f"the oracle port of the reference's algorithm on {len(procs)} single-threaded processes "
                       f"of this host, operators factorised before the timed region "
                       f"({float(np.mean(fact)):.2f} s per process); measured, not extrapolated"),
            "seconds": wall, "per_solve_s": {"median": round(float(np.median(per)), 2),
                                             "max": round(float(np.max(per)), 2)},
            "iterations": {"mean": round(float(np.mean([s[4] for s in solves])), 1),
                           "max": int(max(s[4] for s in solves))},
            "converged": bool(all(s[5] for s in solves))}


def cpu_baseline(n_cols: int, workers: int) -> dict:
    from groundtruth_gb300 import synth
    board = synth.slotted_pair()
    return cpu_pool(cpu_columns(n_cols, len(board.nets), len(board.freqs)), workers, np.asarray(board.freqs))


def run_reference(args):
    """The reference arm: the reference's algorithm on this host's cores (the oracle port; the reference itself
    is pure Python that needs shapely and does not travel).  A warm-up step is a process's setup and
    factorisations; each timed step is one whole column solve, the K columns spread over the band and dealt to
    up to os.cpu_count() single-threaded processes working side by side."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    workers = min(args.steps, os.cpu_count() or 1)
    s = cpu_baseline(args.steps, workers)
    v = s["value"]
    line = {"metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": s["seconds"] / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "solves_per_step": 1, "tol": 1e-10,
                       "step": "one whole column solve; the steps' columns solved side by side on the host cores"},
            "impl": "reference", "cpu_baseline": {**{k: s[k] for k in ("unit", "cores", "kind", "sample")}, "value": v},
            "iterations": s["iterations"], "per_solve_s": s["per_solve_s"], "converged": s["converged"],
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------ GPU side
def replicas_rate(t_step: float, ncol: int, world: int, dist=None, device: str = "cuda") -> tuple:
    """(job step time, whole-job solves/s) of `world` replicas that each solved ncol columns in t_step
    seconds: the slowest replica's time (the max over ranks) is the job's; no data crosses between ranks."""
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([t_step], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_step = float(t.item())
    return t_step, world * ncol / t_step


def run_gpu(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from groundtruth_gb300 import greens, native, stack as gs, synth

    board = synth.slotted_pair()
    if args.nets:
        board.nets = board.nets[: args.nets]
    if args.freqs:
        board.freqs = board.freqs[:: args.freqs]
    t_setup = time.perf_counter()
    st, routes = gs.from_board(board)
    t_setup = time.perf_counter() - t_setup
    # psi of every strip per net on the device (the right-hand sides' setup), beside the host restatement
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for net in board.nets:
        st.handle.strip_coupling(st.sheet_z, st.sheet_t, st.d, net.segments, st.ns)
    psi_dev = (time.perf_counter() - t0) / len(board.nets)
    t0 = time.perf_counter()
    greens.strip_coupling(board.nets[0].segments, [st.xa, st.ya], st.d, st.sheet_z, st.sheet_t)
    psi_host = time.perf_counter() - t0
    lib = st.handle.lib
    freqs = list(board.freqs)
    cols = [(k, q) for k in range(len(routes)) for q in range(len(freqs))]
    ncol = len(cols)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    # operators (factorised Schur complements at every frequency), timed on their own
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ops = st.factorise(freqs, together=True, borrow=args.borrow)
    torch.cuda.synchronize()
    factor_s = time.perf_counter() - t0
    obj = ops[0][0]
    col_op = np.array([ops[q][1] for (_, q) in cols], np.int32)
    rhs_c = np.stack([st.rhs_vector(routes[k].rhs_top(freqs[q]), routes[k].J()) for (k, q) in cols])
    n = st.handle.n_dense
    B = torch.zeros((ncol, n), dtype=torch.complex128, device="cuda")
    X = torch.zeros_like(B)
    st.handle.to_dense(rhs_c, B.data_ptr(), sptr)
    kw = dict(tol=args.tol, restart=args.restart, inner_tol=args.inner_tol, max_its=args.max_its, stream=sptr,
              reorth=args.reorth, outer_k=args.outer_k, precision=args.precision)

    def step():
        return st.handle.solve_device(obj, col_op, B.data_ptr(), X.data_ptr(), **kw)

    for _ in range(max(args.warmup, 0)):
        step()
    clocks = Clocks(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    l0 = lib.gt_launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    its = res = None
    for k in range(args.steps):
        ev[k][0].record(stream)
        its, res = step()
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = int(lib.gt_launch_count() - l0)
    clk = clocks.stop()
    ms = [a.elapsed_time(b) for a, b in ev]
    t_step, value = replicas_rate(float(np.sum(ms)) / args.steps / 1e3, ncol, world, dist, "cuda")

    # accuracy of this run: every column's FP64 residual, and Z_loop against the reference's own full solves
    xc = st.handle.to_compact(X.data_ptr(), ncol, sptr)
    gold = np.load(ROOT / "tests" / "golden" / "slotted_pair_scalars.npz")
    zerr = []
    for k in range(min(2, len(routes))):
        for qg, fg in enumerate(gold["freqs"]):
            if not np.isclose(np.abs(np.asarray(freqs) - fg).min(), 0.0, atol=1e-3 * fg):
                continue
            q = int(np.argmin(np.abs(np.asarray(freqs) - fg)))
            c = cols.index((k, q))
            x = xc[c]
            Vn = np.zeros(st.n_nodes, complex)
            Vn[st.keep] = x[st.nb:]
            sol = routes[k].solution(freqs[q], x[: st.nb], Vn, int(its[c]))
            Zr = complex(gold[f"Z{k}_{qg}"])
            zerr.append(abs(sol.Z_loop - Zr) / abs(Zr))
    # the plane current maps against the reference's own full-size solves of three columns across the band
    ierr = []
    cur = ROOT / "tests" / "golden" / "slotted_pair_currents.npz"
    if cur.exists():
        gc = np.load(cur)
        for n, (k, q) in enumerate(gc["cols"]):
            k, q = int(k), int(q)
            if k >= len(routes) or q >= len(freqs) or not np.isclose(freqs[q], gc["freqs"][q], rtol=1e-9):
                continue
            c = cols.index((k, q))
            x = xc[c]
            Vn = np.zeros(st.n_nodes, complex)
            Vn[st.keep] = x[st.nb:]
            sol = routes[k].solution(freqs[q], x[: st.nb], Vn, int(its[c]))
            got = np.concatenate([np.ravel(sol.I_x), np.ravel(sol.I_y)])
            ref = np.concatenate([np.ravel(gc[f"Ix{n}"]), np.ravel(gc[f"Iy{n}"])]).astype(np.complex128)
            ierr.append(float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))

    # per-kernel-family timing (CUDA events on the launch stream) of one more step
    st.handle.profile(True, levels=args.levels)
    step()
    torch.cuda.synchronize()
    prof = st.handle.profile()
    st.handle.profile(False)
    levels = {k: {"ms": round(v[0], 3), "GBps": round(v[1] / (v[0] * 1e-3) / 1e9, 1)}
              for k, v in prof.items() if ".L" in k}
    prof = {k: v for k, v in prof.items() if ".L" not in k}
    peak, peak_kind = peaks()
    # the roofline's kernel: the longest region that times one kernel (the triangular sweeps' region holds
    # three kernels on four streams, the outer loop's several)
    fam = {k: v for k, v in prof.items() if v[1] > 0 and k.split(".")[0] not in MULTI_KERNEL_REGIONS}
    top = max(fam, key=lambda k: fam[k][0])
    ach = fam[top][1] / (fam[top][0] * 1e-3) / 1e9
    # per launch: the family's algorithmic bytes over its timed regions (one kernel launch of the top kernel
    # each, plus its small partial-sum reduction)
    per_launch = fam[top][1] / max(fam[top][2], 1)
    traffic = round(per_launch * TRAFFIC_RATIO[top]) if top in TRAFFIC_RATIO else None
    prof_total = sum(v[0] for v in prof.values())
    per_family = {k: {"ms": round(v[0], 3), "share": round(v[0] / prof_total, 4),
                      "GBps": round(v[1] / (v[0] * 1e-3) / 1e9, 1) if v[1] > 0 else None, "regions": v[2]}
                  for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}

    # e2e through the C ABI from host buffers: factorise all frequencies + solve + copy out, every step
    e2e_t, e2e_parts = [], []
    # the step's inputs and outputs in page-locked host memory
    # the columns by frequency, so that the sweep's frequency groups are contiguous rows of the host buffers
    by_f = sorted(range(ncol), key=lambda c: (cols[c][1], cols[c][0]))
    key_f = np.array([cols[c][1] for c in by_f])
    rhs_pin = torch.empty(rhs_c.shape, dtype=torch.complex128, pin_memory=True).numpy()
    x_pin = torch.empty(rhs_c.shape, dtype=torch.complex128, pin_memory=True).numpy()
    rhs_pin[...] = rhs_c[by_f]
    skw = dict(restart=args.restart, inner_tol=args.inner_tol, max_its=args.max_its, reorth=args.reorth,
               outer_k=args.outer_k, precision=args.precision)
    sweep = args.e2e_chunks > 1 and not args.borrow
    for k in range(0 if args.no_e2e else max(1, min(args.steps, 2))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        data = [st._freq_tables(f) for f in freqs]
        t1 = time.perf_counter()
        if sweep:       # factorisation of later frequency groups overlapped with the solves of earlier ones
            xh, its2, res2, ok2 = native.solve_sweep(st.handle, freqs, data, key_f, rhs_pin, args.tol,
                                                     chunks=args.e2e_chunks, out=x_pin, **skw)
            t2 = t1
        else:
            ops2 = native.Operators(st.handle, freqs, data, gs.borrow_plan(freqs) if args.borrow else None)
            t2 = time.perf_counter()
            xh, its2, res2, ok2 = native.solve(st.handle, [(ops2, int(q)) for q in key_f], rhs_pin, args.tol,
                                               out=x_pin, **skw)
            del ops2
        e2e_t.append(time.perf_counter() - t0)
        e2e_parts.append({"tables_s": round(t1 - t0, 3),
                          **({"factorise_and_solve_overlapped_s": round(e2e_t[-1] - t1 + t0, 3),
                              "frequency_groups": args.e2e_chunks} if sweep else
                             {"operators_s": round(t2 - t1, 3), "solve_s": round(e2e_t[-1] - t2 + t0, 3)}),
                          "max_rel_residual": float(np.max(res2))})
    e2e = None
    if e2e_t:
        e2e = {"value": world * ncol / float(np.median(e2e_t)), "unit": "solves/s",
               "h2d_bytes_per_step": int(rhs_c.nbytes + sum(sum(np.asarray(a).nbytes for a in d) for d in data)),
               "d2h_bytes_per_step": int(xh.nbytes), "parts": e2e_parts[-1]}

    # plain all-FP64 GPU comparator: one column at a time, FP64 GMRES, same preconditioner
    plain = None
    if not args.no_plain:
        sample = [cols.index((k, q)) for k, q in ((0, 0), (3, 15), (6, 31), (1, 8))]
        t0 = time.perf_counter()
        for c in sample:
            native.solve(st.handle, [ops[cols[c][1]]], rhs_c[c: c + 1], args.tol, restart=args.restart,
                         precision="fp64", max_its=args.max_its, inner_tol=args.tol, outer_k=1, reorth=0.7)
        plain = {"value": len(sample) / (time.perf_counter() - t0), "unit": "solves/s",
                 "sample": "4 columns solved one at a time, FP64 GMRES(50) + FP64 products, operators resident"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        ncpu = min(args.cpu_cols, os.cpu_count() or 1)
        cpu = cpu_baseline(args.cpu_cols, ncpu)
        cpu.pop("seconds")

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "c64 inner / c128 refinement", "data": "synthetic (seeded)",
                "config": {"workload": WORKLOAD, "solves_per_step": ncol, "tol": args.tol, "restart": args.restart,
                           "reorth": args.reorth, "outer_gcr_k": args.outer_k,
                           "parallelism": f"replicas x{world}", "l2": "working set >> L2 (Krylov basis ~48 GB)",
                           "operators": "resident (factorised once, timed separately)"},
                "factorise_s_all_freqs": round(factor_s, 3),
                "iterations": {"mean": float(np.mean(its)), "max": int(np.max(its))},
                "accuracy": {"max_rel_residual": float(np.max(res)),
                             "max_rel_err_Z_vs_reference": float(max(zerr)) if zerr else None,
                             "Z_columns_checked": len(zerr),
                             "max_rel_err_currents_vs_reference": float(max(ierr)) if ierr else None,
                             "current_columns_checked": len(ierr),
                             "currents_note": "relative L2 of the plane current maps (I_x, I_y of both sheets) "
                                              "against the reference's own FP64 solves at rtol 1e-10"},
                "roofline": {"bound": "hbm", "kernel": top, "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                             "frac": round(ach / peak, 4), "peak_kind": peak_kind, "traffic": traffic,
                             "algorithmic_bytes_per_launch": round(per_launch)},
                "setup": {"stack_and_routes_s": round(t_setup, 3), "psi_device_ms_per_net": round(psi_dev * 1e3, 2),
                          "psi_host_ms_per_net": round(psi_host * 1e3, 1)},
                "kernel_families": per_family,
                **({"solve_levels": levels} if levels else {}),
                "e2e": e2e, "gpu_launches": launches // max(args.steps, 1) * args.steps,
                "clocks": clk, "plain_fp64_gpu": plain, "cpu_baseline": cpu}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


# ------------------------------------------------------------------------------------------ what-if edits
def run_what_if(args):
    """Interactive edits on a solved board: each request adds 1-4 stitching vias (60 %), adds a decoupling part
    (20 %) or moves one (20 %: removed, added elsewhere) and answers 1-8 nets at 1-16 of the base's frequencies (whatif.WhatIf: composed from base solves of
    the new branches' injections, or solved on the derived stack).  Requests run one after another; their
    service times also drive a FIFO queue with Poisson arrivals at --rate."""
    import torch
    from groundtruth_gb300 import stack as gs, synth, whatif
    rank = int(os.environ.get("RANK", 0))
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    rng = np.random.default_rng(2024 + rank)
    t0 = time.perf_counter()
    board = synth.what_if_base()
    st, routes = gs.from_board(board)
    setup_s = time.perf_counter() - t0
    wi = whatif.WhatIf(st, routes, board.freqs, tol=board.tol, max_cols=args.max_cols, method=args.what_if_method,
                       border_tol=args.border_tol,
                       restart=args.restart,
                       inner_tol=args.inner_tol, reorth=args.reorth, max_its=args.max_its)
    base_s = wi.baseline()
    n_base = len(routes) * len(board.freqs)
    reqs = []
    for r in range(args.warmup + args.requests):
        u = rng.random()            # 60 % add 1-4 vias, 20 % add a decoupling part, 20 % move one
        vias = u < 0.6
        extra = synth.what_if_branches(board, seed=1000 + r, n_via=int(rng.integers(1, 5)) if vias else 0,
                                       n_part=0 if vias else 1)
        remove = [int(rng.integers(0, st.nbr))] if u >= 0.8 and st.nbr else []
        nets = sorted(int(k) for k in rng.choice(len(routes), size=int(rng.integers(1, 9)), replace=False))
        fq = sorted(int(q) for q in rng.choice(len(board.freqs), size=int(rng.integers(1, 17)), replace=False))
        reqs.append(([gs.Branch(b.a, b.b, b.z, f"edit{r}_{n}", b.kind, b.radius) for n, b in enumerate(extra)],
                     nets, [float(board.freqs[q]) for q in fq], remove))
    from groundtruth_gb300 import native
    lib = native.load()
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", 0)))
    service, cols, its, parts, worst, l0 = [], [], [], [], 0.0, 0
    for r, (br, nets, fq, remove) in enumerate(reqs):
        if r == args.warmup:
            clocks.start()
            l0 = lib.gt_launch_count()
        res = wi.evaluate(br, nets, fq, remove=remove)
        if r < args.warmup:
            continue
        service.append(res.seconds)
        cols.append(len(res.solutions))
        its += res.iterations
        parts.append(res.parts)
        worst = max(worst, max(s.residual for s in res.solutions.values()))
    launches = int(lib.gt_launch_count() - l0)
    ck = clocks.stop()
    sv = np.array(service)
    ms = lambda x: round(float(x) * 1e3, 2)
    line = {
        "metric": "what-if edit latency (p50)", "value": ms(np.median(sv)), "unit": "ms", "n_gpus": 1,
        "higher_is_better": False, "impl": "gb300", "dtype": "c64 inner / c128 outer", "data": "synthetic",
        "config": {"workload": f"what_if_base {board.nx}x{board.ny} @{board.d * 1e3:g}mm GND slot + split PWR, "
                               f"{len(routes)} nets x {len(board.freqs)} freqs; edits: 1-4 vias | add 1 decap | move 1 decap, "
                               "1-8 nets x 1-16 freqs", "tol": board.tol, "max_cols": args.max_cols,
                   "border_tol": args.border_tol},
        "requests": len(sv), "warmup": args.warmup, "p50_ms": ms(np.median(sv)), "p99_ms": ms(np.quantile(sv, 0.99)),
        "mean_ms": ms(sv.mean()), "max_ms": ms(sv.max()), "columns_per_request": float(np.mean(cols)),
        "solves_per_s": round(float(sum(cols) / sv.sum()), 2),
        "sustainable_edits_per_s": round(float(1.0 / sv.mean()), 3),
        "note": "edits one after another (service time); arrivals and batching: --workload serve",
        "iterations_mean": round(float(np.mean(its)), 1), "max_residual": worst,
        "method": args.what_if_method,
        "cold_redo_columns": int(sum(p["cold_redo"] for p in parts)),
        "border_columns": int(sum(p.get("border_columns", 0) for p in parts)),
        "parts_median_s": {k: round(float(np.median([p[k] for p in parts])), 4) for k in parts[0] if k.endswith("_s")},
        "setup": {"stack_and_routes_s": round(setup_s, 2), "baseline_s": round(base_s, 2),
                  "baseline_solves_per_s": round(n_base / base_s, 2)},
        "clocks": ck, "gpu_launches": launches,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------ uneven batch
def run_uneven(args):
    """The uneven-batch workload: --boards seeded boards (sides 64-512, 2-6 layers, cut-outs, stitching vias,
    1-16 nets x 4-16 frequencies; synth.uneven_board), every (net, frequency) of every board solved to the
    boards' tolerance.  Host setup (topology, symbolic analysis, spectra) is outside the timed region; a step
    factorises every board's frequencies and solves all its columns, first one board after another, then with
    --concurrency boards in flight on streams of their own (batch.solve_all); value is the latter's solves/s.
    Each board's result in the mix is checked against its result alone."""
    import torch
    from groundtruth_gb300 import batch, native, synth
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    t0 = time.perf_counter()
    boards = [synth.uneven_board(s) for s in range(args.boards)]
    jobs = batch.prepare(boards)
    setup_s = time.perf_counter() - t0
    nsolve = sum(len(j.cols) for j in jobs)
    smallest = {}
    for j in jobs:                       # warm-up: the kernels' first launches, on the smallest board of each group
        if j.group not in smallest or j.stack.handle.n_dense < smallest[j.group].stack.handle.n_dense:
            smallest[j.group] = j
    for j in smallest.values():
        batch.solve_board(j)
    lib = native.load()
    torch.cuda.synchronize()
    # the mix first: what is left of one-time costs (launch-shape tuning per geometry) falls on it
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    l0 = lib.gt_launch_count()
    t0 = time.perf_counter()
    mixed = batch.solve_all(jobs, concurrency=args.concurrency)
    t_mixed = time.perf_counter() - t0
    launches = int(lib.gt_launch_count() - l0)
    ck = clocks.stop()
    alone, t_alone = None, None
    if not args.no_alone:
        t0 = time.perf_counter()
        alone = batch.solve_all(jobs, concurrency=1)
        t_alone = time.perf_counter() - t0
    dev = max(float(np.linalg.norm(a.x - m.x) / max(np.linalg.norm(a.x), 1e-300)) for a, m in zip(alone, mixed)) \
        if alone else None
    groups = {}
    for j in jobs:
        groups[str(j.group)] = groups.get(str(j.group), 0) + 1
    line = {"metric": "uneven batch solves/s", "value": nsolve / t_mixed, "unit": "solves/s", "n_gpus": 1,
            "steps": 1, "warmup": 1, "ms_per_step": t_mixed * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64 inner / c128 refinement", "data": "synthetic (seeded)",
            "config": {"workload": f"uneven: {args.boards} boards (sides 64-512, 2-6 layers, cut-outs, vias, 1-16 "
                                   "nets x 4-16 log f), factorisation + solve of every column per step",
                       "solves_per_step": nsolve, "tol": boards[0].tol, "concurrency": args.concurrency,
                       "warmup": f"the smallest board of each FFT group ({len(smallest)} boards)",
                       "fft_groups": groups},
            "one_board_at_a_time": {"value": nsolve / t_alone, "unit": "solves/s", "seconds": round(t_alone, 2)}
            if alone else None,
            "max_rel_diff_mix_vs_alone": dev,
            "max_rel_residual": float(max(m.residual.max() for m in mixed)),
            "iterations": {"mean": float(np.mean(np.concatenate([m.its for m in mixed]))),
                           "max": int(max(m.its.max() for m in mixed))},
            "factorise_s_sum": round(sum(m.factorise_s for m in mixed), 2),
            "setup_s": round(setup_s, 1), "gpu_launches": launches, "clocks": ck}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------ largest instance
def run_largest(args):
    """The largest single instance: six plane layers of --side x --side nodes at 0.1 mm (synth.largest_board:
    1024 x 1024 is ~12.4 M strips; 32 nets x 64 frequencies), of which the first --largest-nets nets at
    --largest-freqs frequencies spread over the band are solved.  Host setup (topology, symbolic analysis,
    spectra, right-hand sides) is reported, not timed; the timed step factorises the frequencies (FP32 panels
    kept, one frequency at a time when that is all the memory holds) and solves every column
    (batch.solve_board).  Reported per kernel family: device time, algorithmic GB/s and its fraction of the
    measured HBM bandwidth; per column: the FP64 backward error ||b - Kx|| / ||b|| (the oracle cannot run at this
    size)."""
    import torch
    from groundtruth_gb300 import batch, native, synth
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    t0 = time.perf_counter()
    board = synth.largest_board(args.side)
    nq = len(board.freqs)
    qs = sorted(set(int(round(v)) for v in np.linspace(0, nq - 1, max(1, args.largest_freqs)))) \
        if args.largest_freqs > 1 else [nq // 2]
    board.freqs = np.asarray(board.freqs)[qs]
    board.nets = board.nets[: args.largest_nets]
    job = batch.prepare([board])[0]
    st = job.stack
    setup_s = time.perf_counter() - t0
    lib = native.load()
    torch.cuda.synchronize()
    st.handle.profile(True)
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    l0 = lib.gt_launch_count()
    t0 = time.perf_counter()
    res = batch.solve_board(job)
    torch.cuda.synchronize()
    t_step = time.perf_counter() - t0
    launches = int(lib.gt_launch_count() - l0)
    ck = clocks.stop()
    prof = st.handle.profile()
    st.handle.profile(False)
    peak, peak_kind = peaks()
    fam = {k: {"ms": round(v[0], 1), "GBps": round(v[1] / (v[0] * 1e-3) / 1e9, 1) if v[1] > 0 else None,
               "frac": round(v[1] / (v[0] * 1e-3) / 1e9 / peak, 3) if v[1] > 0 else None, "regions": v[2]}
           for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}
    sym = st.sym
    ncol = len(job.cols)
    line = {"metric": "largest instance solves/s", "value": ncol / t_step, "unit": "solves/s", "n_gpus": 1,
            "steps": 1, "warmup": 0, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64 inner / c128 refinement", "data": "synthetic (seeded)",
            "config": {"workload": f"largest: 6 layers x {args.side}^2 at 0.1 mm, slots + cut-outs + vias; "
                                   f"{len(board.nets)} nets x {len(board.freqs)} f of 32 x 64, factorisation + "
                                   "solve per step", "tol": board.tol, "freqs_hz": [float(f) for f in board.freqs],
                       "strips": int(st.ns), "unknowns": int(st.handle.n_compact), "schur_unknowns": int(sym.n),
                       "panel_entries": int(sym.panel_total), "update_entries": int(sym.upd_total),
                       "largest_front": int(max(sym.nown + sym.nbnd))},
            "seconds": {"setup_untimed": round(setup_s, 1), "factorise": round(res.factorise_s, 1),
                        "step": round(t_step, 1)},
            "backward_error": {"max": float(res.residual.max()), "per_column": [float(r) for r in res.residual]},
            "iterations": {"mean": float(np.mean(res.its)), "max": int(np.max(res.its))},
            "Z_loop": [[float(z.real), float(z.imag)] for z in res.Z],
            "kernel_families": fam, "peak_GBps": peak, "peak_kind": peak_kind, "gpu_launches": launches,
            "clocks": ck}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------ serving
def _serve_requests(board, n_base_branches: int, n: int, seed: int):
    """n what-if requests of the serving workload: a third add 1-4 stitching vias, a third move one decoupling
    part (removed, added elsewhere), a third toggle the slot; each answered on 1-8 nets at 1-16 frequencies."""
    from groundtruth_gb300 import serve, stack as gs, synth
    rng = np.random.default_rng(seed)
    freqs = [float(f) for f in board.freqs]
    out = []
    for r in range(n):
        nets = sorted(int(k) for k in rng.choice(len(board.nets), size=int(rng.integers(1, 9)), replace=False))
        fq = sorted(int(q) for q in rng.choice(len(freqs), size=int(rng.integers(1, 17)), replace=False))
        kind = r % 3
        if kind == 2:
            out.append(serve.Request(nets=nets, freqs=[freqs[q] for q in fq], geometry="toggled"))
            continue
        extra = synth.what_if_branches(board, seed=5000 + r, n_via=int(rng.integers(1, 5)) if kind == 0 else 0,
                                       n_part=0 if kind == 0 else 1)
        out.append(serve.Request(nets=nets, freqs=[freqs[q] for q in fq],
                                 branches=[gs.Branch(b.a, b.b, b.z, f"edit{r}_{m}", b.kind, b.radius)
                                           for m, b in enumerate(extra)],
                                 remove=[int(rng.integers(0, n_base_branches))] if kind == 1 else []))
    return out


def run_serve(args):
    """The serving workload: the 512 x 512 what-if board (GND slot, PWR split, 12 nets x 16 frequencies) and its
    slot-toggled twin resident on the device (spectra, factorisations, base solutions; their setup is reported,
    not timed), and a Poisson stream of --requests what-if requests at --rate per second, each submitted at its
    arrival time to the continuous-batching server (serve.Server) under a --budget-gb device budget.  Latency is
    arrival to answer; throughput is the answered (net, frequency) columns over the stream's span.  The same
    requests served one after another (each waiting for the previous answer) are the serial comparator."""
    import threading
    import torch
    from groundtruth_gb300 import native, serve, stack as gs, synth, whatif
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    t0 = time.perf_counter()
    geos, board = {}, None
    for name, slot in (("base", True), ("toggled", False)):
        b = synth.what_if_base(slot=slot)
        board = board or b
        st, routes = gs.from_board(b)
        st.fp32_panels = name != "base"           # the toggled board takes plain solves only
        # the server's budget sizes its batches (solve_batch still splits what would not fit the device)
        wi = whatif.WhatIf(st, routes, b.freqs, tol=b.tol, max_cols=1 << 20, border_tol=args.border_tol,
                           restart=args.restart, inner_tol=args.inner_tol, reorth=args.reorth, max_its=args.max_its)
        wi.baseline()
        geos[name] = wi
    setup_s = time.perf_counter() - t0
    srv = serve.Server(geos, budget_bytes=args.budget_gb * 1e9, restart=args.restart)
    warm = _serve_requests(board, geos["base"].stack.nbr, max(args.warmup, 1), seed=11)
    for r in warm:
        srv.submit(r).result()
    reqs = _serve_requests(board, geos["base"].stack.nbr, args.requests, seed=12)
    gaps = np.random.default_rng(13).exponential(1.0 / args.rate, len(reqs))
    lib = native.load()
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    l0 = lib.gt_launch_count()
    futs = [None] * len(reqs)
    t_start = time.perf_counter()

    def feed():
        t = t_start
        for i, (r, g) in enumerate(zip(reqs, gaps)):
            t += g
            time.sleep(max(0.0, t - time.perf_counter()))
            r.arrival = time.perf_counter()
            futs[i] = srv.submit(r)
    feeder = threading.Thread(target=feed)
    feeder.start()
    feeder.join()
    answers = [f.result() for f in futs]
    t_end = time.perf_counter()
    launches = int(lib.gt_launch_count() - l0)
    ck = clocks.stop()
    batches = srv.batches[len(warm):]
    lat = np.array([a.latency_s for a in answers])
    ncols = sum(len(a.result.solutions) for a in answers)
    worst = max(c.residual for a in answers for c in a.result.solutions.values())
    # serial: the same requests one after another
    t0 = time.perf_counter()
    serial = []
    for r in reqs:
        r.arrival = 0.0
        a = srv.submit(r).result()
        serial.append(a.latency_s)
    t_serial = time.perf_counter() - t0
    srv.close()
    ms = lambda x: round(float(x) * 1e3, 1)
    line = {"metric": "what-if serving latency p50 / p99 and solves/s", "value": ms(np.median(lat)), "unit": "ms",
            "n_gpus": 1, "higher_is_better": False, "impl": "gb300", "dtype": "c64 inner / c128 refinement",
            "data": "synthetic (seeded)",
            "config": {"workload": f"what_if_base {board.nx}x{board.ny} @{board.d * 1e3:g} mm, GND slot + split PWR, "
                                   f"{len(board.nets)} nets x {len(board.freqs)} f; requests: 1-4 vias | move a decap | "
                                   "toggle the slot, on 1-8 nets x 1-16 f", "rate_per_s": args.rate,
                       "requests": len(reqs), "tol": board.tol, "budget_gb": args.budget_gb,
                       "max_batch_columns": srv.max_cols,
                       "resident_gb": round(srv.resident_bytes / 1e9, 1),
                       "budget": "the requests' working memory; the resident geometries (spectra, factorisations, "
                                 "base solutions) beside it"},
            "p50_ms": ms(np.median(lat)), "p99_ms": ms(np.quantile(lat, 0.99)), "max_ms": ms(lat.max()),
            "solves_per_s": round(ncols / (t_end - t_start), 2), "answered_columns": ncols,
            "span_s": round(t_end - t_start, 2),
            "batches": {"count": len(batches), "requests_mean": round(float(np.mean([b["requests"] for b in batches])), 2),
                        "columns_mean": round(float(np.mean([b["columns"] for b in batches])), 1),
                        "seconds_mean": round(float(np.mean([b["seconds"] for b in batches])), 3)},
            "serial": {"p50_ms": ms(np.median(serial)), "solves_per_s": round(ncols / t_serial, 2),
                       "seconds": round(t_serial, 2)},
            "max_residual_bound": worst, "setup_s": round(setup_s, 1), "gpu_launches": launches, "clocks": ck}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.workload == "serve":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference arm times the headline workload only"}))
            return
        run_serve(args)
        return
    if args.workload == "uneven":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference arm times the headline workload only"}))
            return
        run_uneven(args)
        return
    if args.workload == "largest":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference arm times the headline workload only"}))
            return
        run_largest(args)
        return
    if args.workload == "what_if":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference arm times the headline workload only"}))
            return
        run_what_if(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
