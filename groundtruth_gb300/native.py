"""ctypes binding of the CUDA library's C ABI (include/gt_gb300.h).

``load()`` opens groundtruth_gb300/libgtgb300.so (built in-tree by groundtruth_gb300.build) and fails loudly
when it is missing or no CUDA device is visible: the solver has no CPU path.  ``Geometry`` uploads a
PlaneStack, ``Operators`` factorises frequencies, ``solve`` / ``apply`` run batches."""
from __future__ import annotations

import ctypes as C
import sys
import os
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libgtgb300.so"
GT_OK, GT_NOT_CONVERGED, GT_OUT_OF_MEMORY, GT_TIMEOUT, GT_INVALID_ARGUMENT, GT_DEVICE_ERROR = range(6)

_LIB = None

P = C.c_void_p
I64P = C.POINTER(C.c_int64)
I32P = C.POINTER(C.c_int32)
U8P = C.POINTER(C.c_uint8)
DP = C.POINTER(C.c_double)


def cap_fill_cells(st) -> "np.ndarray | None":
    """gt_geometry_desc.cap_fill of a stack: per cell [n_pairs][nx][ny] of the C segment its capacitance's
    facing copper share (1 elsewhere); None when every cell is whole."""
    t, D = st.top, st.dense
    share = t.cap_share
    if share is None or not len(share) or not np.any(share != 1.0):
        return None
    cells = np.ones(len(t.pair_layers) * t.nx * t.ny)
    cells[D.compact_to_dense[st.ns: st.ns + st.ncap] - D.off_c] = share
    return cells


class GeometryDesc(C.Structure):
    _fields_ = [("n_sheets", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("n_pairs", C.c_int32),
                ("n_branches", C.c_int32), ("precond_sheet", C.c_int32),
                ("n_dense", C.c_int64), ("off_x", C.c_int64), ("off_y", C.c_int64), ("off_c", C.c_int64),
                ("off_b", C.c_int64), ("off_v", C.c_int64),
                ("mask", U8P), ("code_x", U8P), ("code_y", U8P), ("pair_layers", I32P), ("branch_nodes", I32P),
                ("n_compact", C.c_int64), ("compact_to_dense", I64P),
                ("fft_p", C.c_int32 * 4), ("spectrum_x", DP), ("spectrum_y", DP),
                ("n_factor", C.c_int64), ("perm", I64P), ("n_fronts", C.c_int32), ("n_levels", C.c_int32),
                ("level_ptr", I64P), ("front_order", I64P), ("own_start", I64P), ("nown", I64P), ("nbnd", I64P),
                ("bnd_ptr", I64P), ("bnd_idx", I64P), ("child_ptr", I64P), ("child_idx", I64P),
                ("cmap_ptr", I64P), ("cmap_idx", I64P), ("panel_off", I64P), ("upd_off", I64P), ("vec_off", I64P),
                ("panel_total", C.c_int64), ("upd_total", C.c_int64), ("vec_total", C.c_int64),
                ("ent_ptr", I64P), ("ent_row", I32P), ("ent_col", I32P), ("ent_s", I64P),
                ("n_svalues", C.c_int64), ("n_table", C.c_int32), ("sterm_ptr", I64P), ("sterm_tab", I32P),
                ("sterm_coef", DP), ("n_lowrank", C.c_int32),
                ("n_override", C.c_int32), ("override_x", I32P), ("override_y", I32P),
                ("n_narrow", C.c_int64), ("narrow_pos", I64P), ("narrow_sheet", I32P), ("narrow_rdelta", DP),
                ("narrow_dl", DP), ("narrow_ptr", I64P), ("narrow_col", I64P), ("narrow_val", DP),
                ("n_layers", C.c_int32), ("sheet_layer", I32P), ("n_twins", C.c_int32),
                ("narrow_partner", I64P), ("narrow_twin", I32P), ("narrow_twfac", DP),
                ("narrow_rre", DP), ("narrow_twre", DP), ("cap_fill", DP)]


GT_OPS_FP32_PANELS = 1                 # gt_operators_create_ex: keep only the FP32 copies of the factor panels

PRECISIONS = {"mixed": 0, "fp64": 1, "mixed16": 2, "mixed_pc64": 3}

# the library's rule for a stiff factorisation (STIFF_RATIO in api.cu): a branch or capacitance admittance above
# this many times the largest strip admittance, where "mixed" solves apply the preconditioner in FP64
STIFF_RATIO = 4096.0


def stiff_table(tab: np.ndarray, tab_cap0: int) -> bool:
    """Whether an admittance table (strip blocks before tab_cap0, then capacitances and branches) is stiff."""
    tab = np.asarray(tab)
    strip = float(np.abs(tab[:tab_cap0]).max()) if tab_cap0 else 0.0
    tail = float(np.abs(tab[tab_cap0:]).max()) if len(tab) > tab_cap0 else 0.0
    return strip > 0 and tail > STIFF_RATIO * strip


def _precision(name: str) -> int:
    """gt_solve_opts.precision: "mixed" FP32 inner GMRES + FP64 outer, "fp64" all FP64, "mixed16" as "mixed"
    with the Krylov basis stored in FP16, "mixed_pc64" as "mixed" with the preconditioner applied in FP64 (what
    "mixed" becomes by itself on a stiff factorisation)."""
    if name not in PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
    return PRECISIONS[name]


class SolveOpts(C.Structure):
    _fields_ = [("tol", C.c_double), ("restart", C.c_int32), ("max_its", C.c_int32), ("inner_tol", C.c_double),
                ("precision", C.c_int32), ("max_outer", C.c_int32), ("reorth", C.c_double), ("outer_k", C.c_int32),
                ("use_guess", C.c_int32)]


def load():
    """The library, opened once.  Raises ImportError when it is not built, RuntimeError without a GPU."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = Path(os.environ.get("GT_GB300_LIB", LIB_PATH))
    if not path.exists():
        raise ImportError(f"the groundtruth_gb300 CUDA library is not built ({path}); run "
                          "python -m groundtruth_gb300.build")
    lib = C.CDLL(str(path))
    lib.gt_version.restype = C.c_int
    lib.gt_last_error.restype = C.c_char_p
    lib.gt_device_count.restype = C.c_int
    lib.gt_launch_count.restype = C.c_int64
    lib.gt_geometry_create.argtypes = [C.POINTER(GeometryDesc), C.POINTER(P)]
    lib.gt_geometry_free.argtypes = [P]
    lib.gt_geometry_free.restype = None
    lib.gt_geometry_trim.argtypes = [P]
    lib.gt_operators_create.argtypes = [P, C.c_int32, DP, DP, DP, DP, DP, C.POINTER(P)]
    lib.gt_operators_free.argtypes = [P]
    lib.gt_operators_free.restype = None
    lib.gt_solve.argtypes = [P, P, C.c_int32, I32P, DP, C.POINTER(SolveOpts), DP, I32P, DP, P]
    lib.gt_solve_device.argtypes = [P, P, C.c_int32, I32P, P, C.POINTER(SolveOpts), P, I32P, DP, P]
    lib.gt_to_dense.argtypes = [P, C.c_int32, DP, P, P]
    lib.gt_to_compact.argtypes = [P, C.c_int32, P, DP, P]
    lib.gt_apply.argtypes = [P, P, C.c_int32, C.c_int32, C.c_int32, I32P, DP, DP, P]
    lib.gt_profile.argtypes = [P, C.c_char_p, C.c_int32, DP, DP, I32P, C.c_int32]
    lib.gt_strip_coupling.argtypes = [P, DP, DP, C.c_double, C.c_int32, DP, DP, C.POINTER(C.c_int64)]
    lib.gt_node_field.argtypes = [P, C.c_int32, P, C.c_double, P, P, P]
    lib.gt_operators_derive.argtypes = [P, P, C.c_int32, DP, DP, DP, DP, DP, C.POINTER(P)]
    lib.gt_operators_create_shared.argtypes = [P, C.c_int32, DP, DP, DP, DP, DP, I32P, C.POINTER(P)]
    lib.gt_operators_create_ex.argtypes = [P, C.c_int32, DP, DP, DP, DP, DP, I32P, C.c_int32, C.POINTER(P)]
    lib.gt_kernel_spectrum.argtypes = [C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_int32, C.c_int32, DP,
                                       C.c_int32, DP]
    lib.gt_moment.argtypes = [P, C.c_int32, P, DP, C.c_double, DP, P]
    lib.gt_lp_product_noalloc.argtypes = [P, C.c_int32, P, P, P]
    lib.gt_memory.argtypes = [P, C.c_int32, C.POINTER(SolveOpts), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                              C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    if lib.gt_device_count() < 1:
        raise RuntimeError("no CUDA device is visible: the groundtruth_gb300 solver runs on the GPU only")
    _LIB = lib
    return lib


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def check(lib, rc: int, what: str):
    if rc == GT_OK:
        return
    msg = lib.gt_last_error().decode(errors="replace")
    if rc == GT_OUT_OF_MEMORY:
        raise MemoryError(f"{what}: device out of memory ({msg})")
    if rc == GT_INVALID_ARGUMENT:
        raise ValueError(f"{what}: {msg}")
    raise RuntimeError(f"{what} failed (status {rc}): {msg}")


class Geometry:
    """A PlaneStack on the device (gt_geometry_create)."""

    def __init__(self, st):
        lib = load()
        self.lib = lib
        t, D, sym = st.top, st.dense, st.sym
        S, nx, ny = t.S, t.nx, t.ny
        keep_arrays = []

        def arr(x, dtype):
            a = np.ascontiguousarray(x, dtype=dtype)
            keep_arrays.append(a)
            return a

        d = GeometryDesc()
        d.n_sheets, d.nx, d.ny = S, nx, ny
        d.n_pairs, d.n_branches = len(t.pair_layers), t.nbr
        d.precond_sheet = int(st.sheet)
        d.n_dense = D.n
        d.off_x, d.off_y, d.off_c, d.off_b, d.off_v = D.off_x, D.off_y, D.off_c, D.off_b, D.off_v
        d.mask = _ptr(arr(D.mask, np.uint8), C.c_uint8)
        d.code_x = _ptr(arr(st.code["x"], np.uint8), C.c_uint8)
        d.code_y = _ptr(arr(st.code["y"], np.uint8), C.c_uint8)
        d.pair_layers = _ptr(arr(t.pair_layers.reshape(-1), np.int32), C.c_int32)
        node_dense = np.flatnonzero(t.node.ravel())
        d.branch_nodes = _ptr(arr(node_dense[t.branch_ab].reshape(-1) if t.nbr else np.zeros(2), np.int32), C.c_int32)
        d.n_compact = len(D.compact_to_dense)
        d.compact_to_dense = _ptr(arr(D.compact_to_dense, np.int64), C.c_int64)
        for k, v in enumerate((*st.P["x"], *st.P["y"])):
            d.fft_p[k] = v
        d.spectrum_x = _ptr(arr(st.spectrum["x"], np.float64), C.c_double)
        d.spectrum_y = _ptr(arr(st.spectrum["y"], np.float64), C.c_double)
        d.n_factor = sym.n
        d.perm = _ptr(arr(sym.perm, np.int64), C.c_int64)
        d.n_fronts = len(sym.nown)
        d.n_levels = len(sym.level_ptr) - 1
        for name in ("level_ptr", "own_start", "nown", "nbnd", "bnd_ptr", "bnd_idx", "child_ptr", "child_idx",
                     "cmap_ptr", "cmap_idx", "panel_off", "upd_off", "vec_off", "ent_ptr", "ent_s"):
            setattr(d, name, _ptr(arr(getattr(sym, name), np.int64), C.c_int64))
        d.front_order = _ptr(arr(sym.order, np.int64), C.c_int64)
        d.ent_row = _ptr(arr(sym.ent_row, np.int32), C.c_int32)
        d.ent_col = _ptr(arr(sym.ent_col, np.int32), C.c_int32)
        d.panel_total, d.upd_total, d.vec_total = sym.panel_total, sym.upd_total, sym.vec_total
        M = st.sterm
        d.n_svalues = M.shape[0]
        d.n_table = st.n_table
        d.sterm_ptr = _ptr(arr(M.indptr, np.int64), C.c_int64)
        d.sterm_tab = _ptr(arr(M.indices, np.int32), C.c_int32)
        d.sterm_coef = _ptr(arr(M.data, np.float64), C.c_double)
        d.n_lowrank = int(getattr(st, "n_lowrank", 0))
        d.n_override = int(st.n_override)
        if st.n_override:
            d.override_x = _ptr(arr(st.override["x"].reshape(-1), np.int32), C.c_int32)
            d.override_y = _ptr(arr(st.override["y"].reshape(-1), np.int32), C.c_int32)
        nr = st.narrow_rows
        d.n_narrow = len(nr["pos"])
        if d.n_narrow:
            d.narrow_pos = _ptr(arr(nr["pos"], np.int64), C.c_int64)
            d.narrow_sheet = _ptr(arr(nr["sheet"], np.int32), C.c_int32)
            d.narrow_rdelta = _ptr(arr(nr["rdelta"], np.float64), C.c_double)
            d.narrow_dl = _ptr(arr(nr["dl"], np.float64), C.c_double)
            d.narrow_ptr = _ptr(arr(nr["ptr"], np.int64), C.c_int64)
            d.narrow_col = _ptr(arr(nr["col"] if len(nr["col"]) else np.zeros(1), np.int64), C.c_int64)
            d.narrow_val = _ptr(arr(nr["val"] if len(nr["val"]) else np.zeros(1), np.float64), C.c_double)
            if np.any(nr["rre"] != 0) or np.any(nr["twre"] != 0):
                d.narrow_rre = _ptr(arr(nr["rre"], np.float64), C.c_double)
                d.narrow_twre = _ptr(arr(nr["twre"], np.float64), C.c_double)
            if len(st.tw_b):
                d.narrow_partner = _ptr(arr(nr["partner"], np.int64), C.c_int64)
                d.narrow_twin = _ptr(arr(nr["twin"], np.int32), C.c_int32)
                d.narrow_twfac = _ptr(arr(nr["tw_fac"], np.float64), C.c_double)
        d.n_layers = st.N
        d.sheet_layer = _ptr(arr(st.sheet_layer, np.int32), C.c_int32)
        d.n_twins = len(st.twin_parent)
        cells = cap_fill_cells(st)
        if cells is not None:
            d.cap_fill = _ptr(arr(cells, np.float64), C.c_double)
        h = P()
        check(lib, lib.gt_geometry_create(C.byref(d), C.byref(h)), "gt_geometry_create")
        self.h = h
        self.n_dense = D.n
        self.n_compact = len(D.compact_to_dense)

    def __del__(self):
        if getattr(self, "h", None) and _LIB is not None:
            _LIB.gt_geometry_free(self.h)
            self.h = None

    def solve_device(self, obj, col_op: np.ndarray, rhs_ptr: int, x_ptr: int, tol: float, restart: int = 50,
                     max_its: int = 2000, inner_tol: float = 1e-5, precision: str = "mixed", max_outer: int = 40,
                     stream: int = 0, reorth: float = 0.7, outer_k: int = 8):
        """gt_solve_device on dense complex128 device buffers (pointers); returns (its, resid)."""
        idx = np.ascontiguousarray(col_op, np.int32)
        ncol = len(idx)
        its = np.zeros(ncol, np.int32)
        res = np.zeros(ncol)
        o = SolveOpts(tol, restart, max_its, inner_tol, _precision(precision), max_outer, reorth, outer_k, 0)
        rc = self.lib.gt_solve_device(self.h, obj.h, ncol, _ptr(idx, C.c_int32), P(rhs_ptr), C.byref(o), P(x_ptr),
                                      _ptr(its, C.c_int32), _ptr(res, C.c_double), P(stream))
        if rc not in (GT_OK, GT_NOT_CONVERGED):
            check(self.lib, rc, "gt_solve_device")
        return its, res

    def trim(self):
        """gt_geometry_trim: free the solve workspace (reallocated by the next solve)."""
        check(self.lib, self.lib.gt_geometry_trim(self.h), "gt_geometry_trim")

    def to_dense(self, compact: np.ndarray, dense_ptr: int, stream: int = 0):
        c = np.ascontiguousarray(np.atleast_2d(compact), np.complex128)
        check(self.lib, self.lib.gt_to_dense(self.h, c.shape[0], _ptr(c.view(np.float64), C.c_double), P(dense_ptr),
                                             P(stream)), "gt_to_dense")

    def to_compact(self, dense_ptr: int, ncol: int, stream: int = 0) -> np.ndarray:
        out = np.zeros((ncol, self.n_compact), np.complex128)
        check(self.lib, self.lib.gt_to_compact(self.h, ncol, P(dense_ptr), _ptr(out.view(np.float64), C.c_double),
                                               P(stream)), "gt_to_compact")
        return out

    def strip_coupling(self, sheet_z: np.ndarray, sheet_t: np.ndarray, pitch: float, segments: np.ndarray,
                       n_strips: int) -> np.ndarray:
        """psi of every strip on the device (gt_strip_coupling); segments (n, 8) rows (a, b, width, current)."""
        z = np.ascontiguousarray(sheet_z, np.float64)
        t = np.ascontiguousarray(sheet_t, np.float64)
        seg = np.ascontiguousarray(np.asarray(segments, np.float64).reshape(-1, 8))
        psi = np.zeros(max(n_strips, 1))
        ns = C.c_int64(0)
        check(self.lib, self.lib.gt_strip_coupling(self.h, _ptr(z, C.c_double), _ptr(t, C.c_double), float(pitch),
                                                   len(seg), _ptr(seg, C.c_double), _ptr(psi, C.c_double),
                                                   C.byref(ns)), "gt_strip_coupling")
        if ns.value != n_strips:
            raise RuntimeError(f"strip count mismatch: device {ns.value}, host {n_strips}")
        return psi[:n_strips]

    def node_field(self, n_cols: int, x_ptr: int, pitch: float, kx_ptr: int, ky_ptr: int, stream: int = 0):
        """gt_node_field on dense device solutions (pointers)."""
        check(self.lib, self.lib.gt_node_field(self.h, n_cols, P(x_ptr), float(pitch), P(kx_ptr), P(ky_ptr),
                                               P(stream)), "gt_node_field")

    def moment(self, n_cols: int, x_ptr: int, sheet_z: np.ndarray, pitch: float, stream: int = 0) -> np.ndarray:
        """gt_moment on dense device solutions: the plane's part of m per column, (n_cols, 3) complex."""
        z = np.ascontiguousarray(sheet_z, np.float64)
        m = np.zeros((n_cols, 3), np.complex128)
        check(self.lib, self.lib.gt_moment(self.h, n_cols, P(x_ptr), _ptr(z, C.c_double), float(pitch),
                                           _ptr(m.view(np.float64), C.c_double), P(stream)), "gt_moment")
        return m

    def profile(self, on: bool | None = None, levels: bool = False) -> dict:
        """Toggle (on=True/False: reset; levels: time each elimination level too) or read
        {kernel family: (ms, algorithmic bytes, timed regions)}."""
        if on is not None:
            self.lib.gt_profile(self.h, None, 0, None, None, None, (-3 if levels else -2) if on else -1)
            return {}
        cap = 128
        names = C.create_string_buffer(16384)
        ms, by = np.zeros(cap), np.zeros(cap)
        launches = np.zeros(cap, np.int32)
        k = self.lib.gt_profile(self.h, names, 16384, _ptr(ms, C.c_double), _ptr(by, C.c_double),
                                _ptr(launches, C.c_int32), cap)
        keys = names.value.decode().split(",") if k else []
        return {n: (float(ms[i]), float(by[i]), int(launches[i])) for i, n in enumerate(keys)}


class Operators:
    """Factorised Schur complements at several frequencies (gt_operators_create)."""

    def __init__(self, geom: Geometry, keys: list, data: list, factor_of=None, base: "Operators | None" = None,
                 fp32_panels: bool = False):
        """factor_of: optional per-operator index of the operator whose factorisation preconditions it
        (gt_operators_create_shared); None: every operator its own.  base: the base stack's operators at the
        same keys, for a derived geometry (gt_operators_derive: the base's factorisations plus a low-rank
        update for the added branches); kept alive as long as these.  fp32_panels: keep only the FP32 copies of
        the factor (a third of the memory; precision "mixed" / "mixed16" solves only, no derived operators on
        them; a stiff set keeps its FP64 panels anyway)."""
        lib = geom.lib
        self.geom = geom
        w = np.array([x[0] for x in data], np.float64)
        zs = np.ascontiguousarray(np.stack([x[1] for x in data]).astype(np.complex128))
        zc = np.ascontiguousarray(np.stack([x[2] for x in data]).astype(np.complex128)).reshape(len(data), -1)
        zb = np.ascontiguousarray(np.stack([x[3] for x in data]).astype(np.complex128)).reshape(len(data), -1)
        tab = np.ascontiguousarray(np.stack([x[4] for x in data]).astype(np.complex128))
        self._keep = (zs, zc, zb, tab)
        h = P()
        self.base = base
        args = (_ptr(w, C.c_double), _ptr(zs.view(np.float64), C.c_double), _ptr(zc.view(np.float64), C.c_double),
                _ptr(zb.view(np.float64), C.c_double), _ptr(tab.view(np.float64), C.c_double))
        if base is not None:
            if list(keys) != base.keys:
                raise ValueError("derived operators take the base's keys, in its order")
            self.factor_of = base.factor_of
            check(lib, lib.gt_operators_derive(geom.h, base.h, len(data), *args, C.byref(h)), "gt_operators_derive")
        else:
            fo = None if factor_of is None else np.ascontiguousarray(factor_of, np.int32)
            self.factor_of = fo
            check(lib, lib.gt_operators_create_ex(geom.h, len(data), *args,
                                                  None if fo is None else _ptr(fo, C.c_int32),
                                                  GT_OPS_FP32_PANELS if fp32_panels else 0, C.byref(h)),
                  "gt_operators_create_ex")
        self.fp32_panels = bool(fp32_panels) and base is None
        self.h = h
        self.keys = list(keys)

    def __del__(self):
        if getattr(self, "h", None) and _LIB is not None:
            _LIB.gt_operators_free(self.h)
            self.h = None


def _ops_and_index(ops: list):
    """[(Operators, index)] of the columns -> one Operators object and the per-column index into it."""
    objs = {id(o): o for o, _ in ops}
    if len(objs) != 1:
        raise ValueError("all columns of one batch must use operators made together (PlaneStack.factorise)")
    obj = next(iter(objs.values()))
    return obj, np.array([k for _, k in ops], np.int32)


def current_stream() -> int:
    """The calling thread's current PyTorch CUDA stream when torch has initialised CUDA (so that solves issued
    under torch.cuda.stream(s) run on s, beside other streams' work), else 0 (the default stream)."""
    torch = sys.modules.get("torch")
    if torch is not None and torch.cuda.is_available() and torch.cuda.is_initialized():
        return int(torch.cuda.current_stream().cuda_stream)
    return 0


def solve(geom: Geometry, ops: list, rhs: np.ndarray, tol: float, restart: int = 50, max_its: int = 2000,
          inner_tol: float = 1e-5, precision: str = "mixed", max_outer: int = 40, reorth: float = 0.7,
          outer_k: int = 8, x0: np.ndarray | None = None, out: np.ndarray | None = None, stream: int | None = None):
    """rhs: (ncol, n_compact) complex in the reference's order; x0: optional starting points (same shape);
    out: optional C-contiguous complex128 array of that shape to receive x (e.g. page-locked host memory);
    stream: a cudaStream_t (default: current_stream()).  Returns (x, its, resid, converged)."""
    lib = geom.lib
    obj, idx = _ops_and_index(ops)
    rhs = np.ascontiguousarray(rhs, np.complex128)
    ncol = rhs.shape[0]
    if out is not None:
        if out.shape != rhs.shape or out.dtype != np.complex128 or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous complex128 array of the shape of rhs")
        x = out
        x[...] = 0 if x0 is None else x0
    else:
        x = np.zeros_like(rhs) if x0 is None else np.array(x0, np.complex128, order="C", copy=True)
    if x.shape != rhs.shape:
        raise ValueError("x0 must have the shape of rhs")
    its = np.zeros(ncol, np.int32)
    res = np.zeros(ncol)
    o = SolveOpts(tol, restart, max_its, inner_tol, _precision(precision), max_outer, reorth, outer_k,
                  0 if x0 is None else 1)
    st = current_stream() if stream is None else stream
    rc = lib.gt_solve(geom.h, obj.h, ncol, _ptr(idx, C.c_int32), _ptr(rhs.view(np.float64), C.c_double), C.byref(o),
                      _ptr(x.view(np.float64), C.c_double), _ptr(its, C.c_int32), _ptr(res, C.c_double), P(st))
    if rc not in (GT_OK, GT_NOT_CONVERGED):
        check(lib, rc, "gt_solve")
    return x, its, res, res <= tol


def solve_sweep(geom: Geometry, keys: list, tables: list, col_key: np.ndarray, rhs: np.ndarray, tol: float,
                chunks: int = 4, out: np.ndarray | None = None, stream: int | None = None, fp32_panels: bool = False,
                **solve_kw):
    """A frequency sweep from host buffers, its factorisation overlapped with its solves: the operators (keys,
    tables as for Operators) are made in `chunks` contiguous groups of frequencies by a second host thread,
    each group on a stream of its own (gt_operators_create_ex takes no geometry lock), while the columns of
    the groups already made are solved on `stream` (gt_solve).  The FP64 factorisation (the FP64 pipes, few SMs
    at the top of the elimination tree) so runs beside the FP32 solve instead of before it.  Column c of rhs
    is at frequency index col_key[c]; the columns of a group must be contiguous rows of rhs (sort them by
    frequency), so that page-locked rhs and out pass to each solve as views.  Returns (x, its, resid,
    converged) like solve."""
    import threading
    rhs = np.asarray(rhs)
    col_key = np.asarray(col_key)
    nq, ncol = len(keys), rhs.shape[0]
    bounds = np.linspace(0, nq, max(1, min(chunks, nq)) + 1).round().astype(int)
    groups = [range(bounds[i], bounds[i + 1]) for i in range(len(bounds) - 1) if bounds[i + 1] > bounds[i]]
    group_of = np.empty(nq, np.int64)
    for gi, g in enumerate(groups):
        group_of[list(g)] = gi
    gcol = group_of[col_key]
    if np.any(np.diff(gcol) < 0):
        raise ValueError("the columns must be sorted by their frequency's group")
    x = out if out is not None else np.zeros(rhs.shape, np.complex128)
    its = np.zeros(ncol, np.int32)
    res = np.zeros(ncol)
    made = [None] * len(groups)
    ready = [threading.Event() for _ in groups]
    failed = []

    def factorise():
        try:
            for gi, g in enumerate(groups):
                made[gi] = Operators(geom, [keys[q] for q in g], [tables[q] for q in g], fp32_panels=fp32_panels)
                ready[gi].set()
        except BaseException as e:          # handed to the solving thread
            failed.append(e)
            for r in ready:
                r.set()

    th = threading.Thread(target=factorise, name="sweep factorisation", daemon=True)
    th.start()
    try:
        for gi, g in enumerate(groups):
            ready[gi].wait()
            if failed:
                raise failed[0]
            sel = np.flatnonzero(gcol == gi)
            if not len(sel):
                made[gi] = None
                continue
            a, b = int(sel[0]), int(sel[-1]) + 1
            ops = [(made[gi], int(col_key[c]) - g.start) for c in range(a, b)]
            _, its[a:b], res[a:b], _ = solve(geom, ops, rhs[a:b], tol, out=x[a:b], stream=stream, **solve_kw)
            made[gi] = None                 # the group's factorisations go before the next group's solve
    finally:
        th.join()
    return x, its, res, res <= tol


def memory(geom: Geometry, n_cols: int, restart: int = 50, precision: str = "mixed", outer_k: int = 8) -> dict:
    """gt_memory: {"need": bytes a solve of n_cols columns allocates, "held": the geometry's workspace now,
    "free" / "total": the device's}."""
    o = SolveOpts(1e-5, restart, 1, 1e-5, _precision(precision), 1, 0.0, outer_k, 0)
    v = [C.c_int64(0) for _ in range(4)]
    check(geom.lib, geom.lib.gt_memory(geom.h, int(n_cols), C.byref(o), *(C.byref(x) for x in v)), "gt_memory")
    return dict(zip(("need", "held", "free", "total"), (x.value for x in v)))


def kernel_spectrum(n_axial: int, n_lateral: int, d: float, dz: float, P0: int, P1: int,
                    near: np.ndarray) -> np.ndarray:
    """The strip kernel's real spectrum quadrant (P0/2+1, P1/2+1) computed on the device (gt_kernel_spectrum);
    near: (n, n) tape-integrated values at the nearest offsets."""
    lib = load()
    nr = np.ascontiguousarray(near, np.float64)
    out = np.zeros((P0 // 2 + 1, P1 // 2 + 1))
    check(lib, lib.gt_kernel_spectrum(int(n_axial), int(n_lateral), float(d), float(dz), int(P0), int(P1),
                                      _ptr(nr, C.c_double), nr.shape[0], _ptr(out, C.c_double)), "gt_kernel_spectrum")
    return out


def apply(geom: Geometry, obj: Operators, kind: str, x: np.ndarray, op_index, precision: str = "fp64") -> np.ndarray:
    """One operator application on compact vectors: kind "matvec", "precond" or "lp"."""
    lib = geom.lib
    x = np.ascontiguousarray(np.atleast_2d(x), np.complex128)
    ncol = x.shape[0]
    idx = np.ascontiguousarray(np.broadcast_to(np.asarray(op_index, np.int32), (ncol,)))
    y = np.zeros_like(x)
    k = {"matvec": 0, "precond": 1, "lp": 2}[kind]
    rc = lib.gt_apply(geom.h, obj.h, k, 1 if precision == "fp64" else 0, ncol, _ptr(idx, C.c_int32),
                      _ptr(x.view(np.float64), C.c_double), _ptr(y.view(np.float64), C.c_double), None)
    check(lib, rc, "gt_apply")
    return y
