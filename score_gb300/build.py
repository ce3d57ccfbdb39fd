"""Build the in-tree native libraries (score_gb300/_lib/).

libscore_gb300.so  the CUDA sm_103a growth step and its host engine, plus the host
                   entry points (.uds parameters, host mobility weight, generator);
libscore_host.so   the host entry points alone (no CUDA): input preparation for the
                   CPU timing of the reference's algorithm, which must not load the
                   CUDA library.

Both are built next to the package so the process that uses them loads them from the
source tree.  The translation units compile in parallel; -ffp-contract=off /
-fmad=false keep FP64 rounding identical to the reference's x86/aarch64 builds (no
fused multiply-add contraction anywhere).
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
HOSTLIB = "libscore_host.so"
HOST_SRCS = ("host_api.cpp", "host_model.cpp", "host_generate.cpp")  # the host-only library's sources
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


def host_library_path() -> Path:
    return LIBDIR / HOSTLIB


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile libscore_gb300.so and libscore_host.so if any source is newer than them;
    return the CUDA library's path."""
    out = library_path()
    hout = host_library_path()
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    deps = srcs + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [HERE.parent / "include" / "score_gb300.h"]
    if not force and all(o.exists() and all(o.stat().st_mtime >= p.stat().st_mtime for p in deps) for o in (out, hout)):
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
    htmp = hout.with_suffix(".so.tmp")
    _run([nvcc, "-shared", "-o", str(htmp), *[str(objdir / (Path(n).stem + ".o")) for n in HOST_SRCS], "-lpthread"])
    os.replace(htmp, hout)
    return out


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(p)
