"""Build of the sm_103a CUDA library libdsplat_gb300.so (the C ABI of include/dsplat_gb300.h).

Each csrc/*.cu file is compiled by nvcc in parallel, then linked with cuBLAS into
dsplat/_build/libdsplat_gb300.so. A rebuild happens only when a source or the
header is newer than the library. No torch headers are involved: the library
takes plain device pointers, and kernels/_lib.py binds it with ctypes.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
SOURCES = PACKAGE / "csrc"
OUTPUT = PACKAGE / "_build"
LIBRARY = OUTPUT / "libdsplat_gb300.so"
INCLUDE = PACKAGE.parent.parent / "include"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    candidate = Path(home) / "bin" / "nvcc"
    if candidate.exists():
        return str(candidate)
    found = shutil.which("nvcc")
    if found is None:
        raise RuntimeError("nvcc not found: set CUDA_HOME or put nvcc on PATH")
    return found


def _flags(verbose_ptxas: bool) -> list[str]:
    flags = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INCLUDE}",
             f"-I{SOURCES}"]
    if verbose_ptxas:
        flags += ["-Xptxas", "-v"]
    return flags


def _stale() -> bool:
    if not LIBRARY.exists():
        return True
    built = LIBRARY.stat().st_mtime
    inputs = list(SOURCES.glob("*.cu")) + list(SOURCES.glob("*.cuh")) + [INCLUDE / "dsplat_gb300.h"]
    return any(path.stat().st_mtime > built for path in inputs)


def build(force: bool = False, verbose_ptxas: bool = False, jobs: int | None = None) -> Path:
    """Compile and link the library if needed; returns its path."""
    if not force and not _stale():
        return LIBRARY
    OUTPUT.mkdir(exist_ok=True)
    nvcc = _nvcc()
    sources = sorted(SOURCES.glob("*.cu"))

    def compile_one(source: Path) -> tuple[Path, str]:
        obj = OUTPUT / (source.stem + ".o")
        cmd = [nvcc, *_flags(verbose_ptxas), "-c", str(source), "-o", str(obj)]
        done = subprocess.run(cmd, capture_output=True, text=True)
        if done.returncode != 0:
            raise RuntimeError(f"nvcc failed on {source.name}:\n{done.stderr}")
        return obj, done.stderr

    with ThreadPoolExecutor(max_workers=jobs or min(8, len(sources))) as pool:
        results = list(pool.map(compile_one, sources))
    if verbose_ptxas:
        for _, log in results:
            sys.stderr.write(log)
    home = Path(nvcc).resolve().parent.parent
    temporary = LIBRARY.with_suffix(".so.tmp")
    link = [nvcc, ARCH, "-shared", "-o", str(temporary), *[str(obj) for obj, _ in results],
            f"-L{home / 'lib64'}", "-lcublas"]
    done = subprocess.run(link, capture_output=True, text=True)
    if done.returncode != 0:
        raise RuntimeError(f"link failed:\n{done.stderr}")
    os.replace(temporary, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
