"""The C ABI library loads and exports every entry point include/gt_gb300.h declares (no GPU needed)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared():
    text = (ROOT / "include" / "gt_gb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|void|const char\*)\s+(gt_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    from groundtruth_gb300 import build
    path = build.build()
    return ctypes.CDLL(str(path))


def test_every_declared_symbol_is_exported(lib):
    names = declared()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n


def test_version_and_error_text_without_a_device(lib):
    lib.gt_version.restype = ctypes.c_int
    lib.gt_last_error.restype = ctypes.c_char_p
    assert lib.gt_version() >= 100
    assert isinstance(lib.gt_last_error(), bytes)


def test_solver_refuses_to_run_without_the_library(monkeypatch, tmp_path):
    from groundtruth_gb300 import native
    monkeypatch.setattr(native, "_LIB", None)
    monkeypatch.setenv("GT_GB300_LIB", str(tmp_path / "missing.so"))
    with pytest.raises(ImportError):
        native.load()


GT_INVALID_ARGUMENT = 4


def _refused(lib, rc, text):
    lib.gt_last_error.restype = ctypes.c_char_p
    assert rc == GT_INVALID_ARGUMENT
    assert text in lib.gt_last_error().decode()


def test_malformed_geometries_are_refused_before_any_device_call(lib):
    """gt_geometry_create's argument checks (PlaneStack.__init__'s SolverError / ValueError, peec.py:1559-1593):
    the ones that come before its first device allocation, so they run here without a GPU."""
    from groundtruth_gb300 import native
    lib.gt_geometry_create.restype = ctypes.c_int
    out = ctypes.c_void_p()
    _refused(lib, lib.gt_geometry_create(None, ctypes.byref(out)), "null argument")
    d = native.GeometryDesc()
    d.nx = d.ny = 10
    d.fft_p[:] = [16, 16, 16, 16]
    for s in (0, 7):
        d.n_sheets = s
        _refused(lib, lib.gt_geometry_create(ctypes.byref(d), ctypes.byref(out)), "1 to 6 sheets")
    d.n_sheets = 2
    d.nx = 2
    _refused(lib, lib.gt_geometry_create(ctypes.byref(d), ctypes.byref(out)), "at least 3 x 3")
    d.nx = 10
    for bad in (20, 4, 40, 0):
        d.fft_p[2] = bad
        _refused(lib, lib.gt_geometry_create(ctypes.byref(d), ctypes.byref(out)), "FFT sizes")
    d.fft_p[2] = 24
    d.n_layers = 3
    _refused(lib, lib.gt_geometry_create(ctypes.byref(d), ctypes.byref(out)), "n_layers must not exceed")
    d.n_sheets, d.n_layers = 3, 2
    _refused(lib, lib.gt_geometry_create(ctypes.byref(d), ctypes.byref(out)), "sheet_layer needed")
    layers = (ctypes.c_int32 * 3)(0, 1, 2)
    d.sheet_layer = ctypes.cast(layers, native.I32P)
    _refused(lib, lib.gt_geometry_create(ctypes.byref(d), ctypes.byref(out)), "sheet_layer out of range")
    assert out.value is None


def test_calls_without_a_geometry_are_refused(lib):
    """Every entry point that takes a geometry or operators refuses a null one (and other malformed sizes) with
    GT_INVALID_ARGUMENT and a message, before touching the device."""
    P, N = ctypes.c_void_p, None
    one = (ctypes.c_double * 8)()
    out = ctypes.c_void_p()
    calls = [
        ("gt_operators_create", (N, 1, one, one, one, one, one, ctypes.byref(out))),
        ("gt_operators_create_shared", (N, 1, one, one, one, one, one, N, ctypes.byref(out))),
        ("gt_operators_derive", (N, N, 1, one, one, one, one, one, ctypes.byref(out))),
        ("gt_solve", (N, N, 1, N, one, N, N, one, N, N)),
        ("gt_solve_device", (N, N, 1, N, P(1), N, P(1), N, N, N)),
        ("gt_memory", (N, 1, N, N, N, N, N)),
        ("gt_apply", (N, N, 0, 0, 1, N, P(1), P(1), N)),
        ("gt_strip_coupling", (N, one, one, ctypes.c_double(1e-3), 0, N, one, N)),
        ("gt_node_field", (N, 1, P(1), ctypes.c_double(1e-3), P(1), P(1), N)),
        ("gt_moment", (N, 1, P(1), one, ctypes.c_double(1e-3), one, N)),
    ]
    for name, args in calls:
        fn = getattr(lib, name)
        fn.restype = ctypes.c_int
        _refused(lib, fn(*args), "bad arguments")
    lib.gt_kernel_spectrum.restype = ctypes.c_int
    quad = (ctypes.c_double * 64)()
    d, dz = ctypes.c_double(1e-3), ctypes.c_double(0.0)
    _refused(lib, lib.gt_kernel_spectrum(0, 4, d, dz, 16, 16, one, 1, quad), "bad arguments")
    _refused(lib, lib.gt_kernel_spectrum(4, 4, d, dz, 20, 16, one, 1, quad), "FFT sizes")
    _refused(lib, lib.gt_kernel_spectrum(12, 4, d, dz, 16, 16, one, 1, quad), "cover 2n - 1")


def _c_struct(name: str) -> list:
    """(field, bytes) of a typedef'd struct in include/gt_gb300.h, in declaration order."""
    text = (ROOT / "include" / "gt_gb300.h").read_text()
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    sizes = {"int32_t": 4, "int64_t": 8, "double": 8, "uint8_t": 1}
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        m = re.match(r"(?:const\s+)?(\w+)\s*(\*?)\s*(.*)", decl)
        ctype, ptr, names = m.groups()
        for nm in names.split(","):
            nm = nm.strip().lstrip("*")
            arr = re.match(r"(\w+)\[(\d+)\]", nm)
            if arr:
                out.append((arr.group(1), sizes[ctype] * int(arr.group(2))))
            else:
                out.append((nm, 8 if ptr or "*" in decl.split(nm)[0] else sizes[ctype]))
    return out


def test_the_ctypes_descriptors_match_the_header():
    """native.GeometryDesc and SolveOpts have the header's fields, in its order and of its sizes (the ABI the
    library reads them by)."""
    import ctypes as C
    from groundtruth_gb300 import native
    for struct, cls in (("gt_geometry_desc", native.GeometryDesc), ("gt_solve_opts", native.SolveOpts)):
        header = _c_struct(struct)
        ours = [(f[0], C.sizeof(f[1])) for f in cls._fields_]
        assert ours == header, struct
