"""Build ``libdgfem_gb300.so`` in-tree with nvcc for sm_103a.

Each ``.cu`` file is compiled to an object in parallel, then linked into one
shared library next to the package (``actx_dgfem_suite_gb300/libdgfem_gb300.so``).
The CUDA runtime is linked statically so the library has no dependency on a
particular ``libcudart`` soname.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

CSRC = Path(__file__).resolve().parent
PKG = CSRC.parent
LIB_NAME = "libdgfem_gb300.so"
LIB_PATH = PKG / LIB_NAME
BUILD_DIR = PKG / "_build"
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required")
    return cand


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _deps() -> list[Path]:
    return (_sources() + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h"))
            + [PKG.parent / "include" / "dgfem_gb300.h"])


def is_stale() -> bool:
    if not LIB_PATH.exists():
        return True
    t = LIB_PATH.stat().st_mtime
    return any(p.stat().st_mtime > t for p in _deps())


def build(force: bool = False, verbose: bool = False,
          extra_flags: list[str] | None = None) -> Path:
    if not force and not is_stale():
        return LIB_PATH
    BUILD_DIR.mkdir(exist_ok=True)
    cc = nvcc()
    flags = ARCH_FLAGS + NVCC_FLAGS + (extra_flags or [])

    def compile_one(src: Path) -> Path:
        obj = BUILD_DIR / (src.stem + ".o")
        cmd = [cc, *flags, "-c", str(src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr)
        return obj

    srcs = _sources()
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [cc, *ARCH_FLAGS, "-shared", "-cudart", "static",
           *[str(o) for o in objs], "-o", str(tmp)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    import sys
    p = build(force="--force" in sys.argv, verbose=True)
    print(p)
