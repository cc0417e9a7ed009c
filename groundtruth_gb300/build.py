"""Build the CUDA library in-tree: groundtruth_gb300/libgtgb300.so for sm_103a (GB300).

    python -m groundtruth_gb300.build          (or __graft_entry__.build())

Each translation unit is compiled in parallel with nvcc, then linked into one shared library exporting the
C ABI of include/gt_gb300.h.  Objects go to groundtruth_gb300/_build/."""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
SRC = HERE / "csrc"
OUT = HERE / "libgtgb300.so"
OBJ = HERE / "_build"
UNITS = ["api.cu", "lp.cu", "stencil.cu", "factor.cu", "gmres.cu", "noalloc.cu", "coupling.cu", "outputs.cu", "spectra.cu", "woodbury.cu", "narrow.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{ROOT / 'include'}",
         "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src] + list(SRC.glob("*.cuh")) + list(SRC.glob("*.h")) + [ROOT / "include" / "gt_gb300.h"]
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, extra: list | None = None) -> Path:
    OBJ.mkdir(exist_ok=True)
    cc = nvcc()
    flags = FLAGS + list(extra or [])

    def one(unit: str):
        src, obj = SRC / unit, OBJ / (unit + ".o")
        if not _stale(obj, src) and not extra:
            return obj, ""
        cmd = [cc, *ARCH, *flags, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {unit}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with ThreadPoolExecutor(len(UNITS)) as ex:
        results = list(ex.map(one, UNITS))
    for obj, err in results:
        if verbose and err:
            print(err, file=sys.stderr)
    objs = [str(o) for o, _ in results]
    if not OUT.exists() or any(Path(o).stat().st_mtime > OUT.stat().st_mtime for o in objs) or extra:
        tmp = OUT.with_suffix(".so.tmp")
        r = subprocess.run([cc, *ARCH, "-shared", "-o", str(tmp), *objs, "-lcudart"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
