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
