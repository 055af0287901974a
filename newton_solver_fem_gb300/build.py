"""Build ``libfemgb300.so`` in-tree with nvcc for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled to an object in parallel, then
linked into one shared library next to this file.  No torch headers are used:
the library's interface is the C ABI in ``include/fem_gb300.h``.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
ROOT = PACKAGE.parent
CSRC = PACKAGE / "csrc"
BUILD = PACKAGE / "_build"
LIBRARY = PACKAGE / "libfemgb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    found = shutil.which("nvcc")
    if found:
        return found
    candidate = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if candidate.exists():
        return str(candidate)
    raise RuntimeError("nvcc not found; set CUDA_HOME")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False, force: bool = False) -> Path:
    """Compile (if stale) and return the path of the shared library."""
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + [ROOT / "include" / "fem_gb300.h"]
    compiler = nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.stem + ".o")
        if force or ptxas_info or _stale(obj, [src, *headers]):
            cmd = [compiler, *ARCH, *FLAGS, *extra, "-I", str(ROOT / "include"), "-I", str(CSRC), "-c", str(src),
                   "-o", str(obj)]
            if verbose:
                print(" ".join(cmd), flush=True)
            res = subprocess.run(cmd, capture_output=True, text=True)
            if res.returncode != 0:
                raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
            if verbose or ptxas_info:
                sys.stdout.write(res.stdout + res.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as pool:
        objects = list(pool.map(compile_one, sources()))
    if force or _stale(LIBRARY, objects):
        cmd = [compiler, *ARCH, "-shared", "-cudart", "static", "-o", str(LIBRARY), *map(str, objects)]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    return LIBRARY


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv, force="--force" in sys.argv)
    print(LIBRARY)
