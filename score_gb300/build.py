"""Build the in-tree native library libscore_gb300.so (CUDA sm_103a + host C++).

The library is built next to the package (score_gb300/_lib/) so the process that
uses it loads it from the source tree.  Three translation units compile in
parallel; -ffp-contract=off / -fmad=false keep FP64 rounding identical to the
reference's x86/aarch64 builds (no fused multiply-add contraction anywhere).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
LIBDIR = HERE / "_lib"
LIBNAME = "libscore_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build score_gb300")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def library_path() -> Path:
    return LIBDIR / LIBNAME


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile libscore_gb300.so if any source is newer than it; return its path."""
    out = library_path()
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    deps = srcs + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [HERE.parent / "include" / "score_gb300.h"]
    if not force and out.exists() and all(out.stat().st_mtime >= p.stat().st_mtime for p in deps):
        return out
    LIBDIR.mkdir(exist_ok=True)
    nvcc = nvcc_path()
    objdir = LIBDIR / "obj"
    objdir.mkdir(exist_ok=True)
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", str(HERE.parent / "include")]
    jobs = []
    for s in srcs:
        o = objdir / (s.stem + ".o")
        if s.suffix == ".cu":
            cmd = [nvcc, *ARCH, "-lineinfo", "-fmad=false", "-Xptxas", "-v" if verbose else "-O3", *common, "-c", str(s), "-o", str(o)]
        else:
            cmd = [nvcc, "-x", "c++", *common, "-c", str(s), "-o", str(o)]
        jobs.append((cmd, o))
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(lambda j: _run(j[0]), jobs))
    tmp = out.with_suffix(".so.tmp")
    _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *[str(o) for _, o in jobs], "-lcudart", "-lpthread"])
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(p)
