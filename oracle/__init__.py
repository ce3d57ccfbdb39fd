"""CPU oracle of the SCORE growth step — TEST INFRASTRUCTURE ONLY.

Two checkers live here; only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline use them, and never as the thing measured or shipped:

* ``run`` — the plain-C restatement in score_oracle.c (single-threaded FP64).
* ``run_ref`` — the SCORE reference itself, compiled from its own sources by
  oracle/ref/Makefile into oracle/_ref/ (only where the reference sources exist),
  driven by oracle/ref/score_ref_driver.cpp.

The restatement is pinned against the reference run here and against the
golden fixtures in tests/golden/ that the reference produced.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REFOUT = HERE / "_ref"
# the reference's source tree: only from $SCORE_REFERENCE (no default location); without
# it, the harness prebuilt into oracle/_ref/ is used when present
REFERENCE_SRC = Path(os.environ["SCORE_REFERENCE"]) if os.environ.get("SCORE_REFERENCE") else None

STEP_DTYPE = np.dtype([("step", "<u4"), ("n_nuclei", "<u4"), ("t", "<f8"), ("dt", "<f8"), ("dt_used", "<f8"),
                       ("Xcells", "<f8"), ("X", "<f8"), ("Sv", "<u8"), ("n_full", "<u8"), ("n_new", "<u8"),
                       ("Pmax", "<f8"), ("rhomax", "<f8"), ("dXstep", "<f8"), ("next_never", "<u4", 2),
                       ("n_recycled", "<u4", 2)])
REF_STEP_DTYPE = np.dtype([("step", "<u4"), ("pad", "<u4"), ("t", "<f8"), ("dt", "<f8"), ("Xcells", "<f8"),
                           ("Sv", "<u8"), ("nfull", "<u8"), ("Pmax", "<f8"), ("rhomax", "<f8"), ("dXstep", "<f8")])


class OracleOut(C.Structure):
    _fields_ = [("n_steps", C.c_uint32), ("status", C.c_int), ("dt0", C.c_double), ("Pmax0", C.c_double),
                ("n_nuclei", C.c_uint32), ("seconds", C.c_double)]


def build_oracle(force: bool = False) -> Path:
    out = BUILD / "liboracle.so"
    src = [HERE / "score_oracle.c", HERE / "score_oracle.h", HERE.parent / "include" / "score_gb300.h"]
    if not force and out.exists() and all(out.stat().st_mtime >= s.stat().st_mtime for s in src):
        return out
    BUILD.mkdir(exist_ok=True)
    tmp = out.with_suffix(".tmp.so")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=gnu11", str(HERE / "score_oracle.c"),
                    "-o", str(tmp), "-lm"], check=True)
    os.replace(tmp, out)
    return out


def reference_sources() -> bool:
    """True when $SCORE_REFERENCE points at the reference's source tree."""
    return REFERENCE_SRC is not None and (REFERENCE_SRC / "src" / "SCORE_Kernel.cpp").exists()


def reference_available() -> bool:
    return reference_sources() or (REFOUT / "score_ref_driver").exists()


def build_ref() -> Path | None:
    """Compile the reference harness from $SCORE_REFERENCE; without the sources, the
    prebuilt harness in oracle/_ref/ if there is one, else None ("reference sources not
    found")."""
    exe = REFOUT / "score_ref_driver"
    if not reference_sources():
        return exe if exe.exists() else None
    subprocess.run(["make", "-s", "-C", str(HERE / "ref"), f"REF={REFERENCE_SRC}", f"-j{os.cpu_count() or 4}"], check=True)
    return exe


_lib = None


def _load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(build_oracle()))
        lib.oracle_run.restype = C.c_int
        lib.oracle_mobility_weight.restype = C.c_double
        lib.oracle_mobility_weight.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.oracle_create.restype = C.c_void_p
        lib.oracle_advance.restype = C.c_int
        lib.oracle_advance.argtypes = [C.c_void_p, C.c_double, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p]
        lib.oracle_done.restype = C.c_int
        lib.oracle_done.argtypes = [C.c_void_p, C.c_double]
        lib.oracle_finish.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.oracle_destroy.argtypes = [C.c_void_p]
        lib.oracle_time.restype = C.c_double
        lib.oracle_time.argtypes = [C.c_void_p]
        lib.oracle_log_count.restype = C.c_uint32
        lib.oracle_log_count.argtypes = [C.c_void_p]
        lib.oracle_log_get.restype = C.c_int
        lib.oracle_log_get.argtypes = [C.c_void_p, C.c_uint32] + [C.c_void_p] * 6
        lib.oracle_binarize.argtypes = [C.c_void_p, C.c_void_p]
        lib.oracle_percolation.restype = C.c_int
        lib.oracle_percolation.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int] + [C.c_void_p] * 6
        lib.oracle_interp_count.restype = C.c_double
        lib.oracle_interp_count.argtypes = [C.c_void_p, C.c_uint32, C.c_double]
        lib.oracle_rediscr_kinetics.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.oracle_rediscr_macrotexture.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def run(params, domain, ptable=None, x_target: float = -1.0, max_steps: int = 0, trace_cap: int = 200000) -> dict:
    """Run nucleation + growth on the CPU restatement; returns trace, labels, counts, summary."""
    lib = _load()
    d = domain
    trace = np.zeros(trace_cap, dtype=STEP_DTYPE)
    labels = np.empty(d.ncells, dtype=np.uint32)
    rc = np.empty(max(d.nrxg, 1), dtype=np.uint32)
    dc = np.empty(d.ndefg, dtype=np.uint32)
    out = OracleOut()
    arrs = [np.ascontiguousarray(x) for x in (d.grid, d.defg_quat, d.defg_rho0, d.rxg_quat, d.rxg_site, d.rxg_tincub)]
    pt = None if ptable is None else np.ascontiguousarray(ptable, dtype=np.float64)
    s = lib.oracle_run(C.byref(params), _p(arrs[0]), _p(arrs[1]), _p(arrs[2]), C.c_uint32(d.ndefg), _p(arrs[3]), _p(arrs[4]),
                       _p(arrs[5]), C.c_uint32(d.nrxg), _p(pt), C.c_double(x_target), C.c_uint32(max_steps), _p(trace),
                       C.c_uint32(trace_cap), _p(labels), _p(rc), _p(dc), C.byref(out))
    n = min(out.n_steps, trace_cap)
    return {"status": s, "trace": trace[:n], "labels": labels, "rxg_counts": rc[: d.nrxg], "defg_counts": dc,
            "dt0": out.dt0, "Pmax0": out.Pmax0, "n_nuclei": out.n_nuclei, "seconds": out.seconds, "n_steps": out.n_steps}


class Sim:
    """One oracle run advanced in pieces (bounded CPU samples of a long run).

    ``advance(x_target, max_steps)`` runs the step loop until the stop rule with
    ``x_target`` holds or ``max_steps`` more steps are done, and returns this piece's
    trace rows and loop seconds; pieces concatenate to exactly the trace of ``run``."""

    def __init__(self, params, domain, ptable=None):
        self._lib = _load()
        d = domain
        self.params = params
        self.ncells, self.nrxg, self.ndefg = d.ncells, d.nrxg, d.ndefg
        self._keep = [np.ascontiguousarray(x) for x in (d.grid, d.defg_quat, d.defg_rho0, d.rxg_quat, d.rxg_site, d.rxg_tincub)]
        self._pt = None if ptable is None else np.ascontiguousarray(ptable, dtype=np.float64)
        k = self._keep
        self._h = self._lib.oracle_create(C.byref(params), _p(k[0]), _p(k[1]), _p(k[2]), C.c_uint32(d.ndefg), _p(k[3]), _p(k[4]),
                                          _p(k[5]), C.c_uint32(d.nrxg), _p(self._pt))
        if not self._h:
            raise MemoryError("oracle_create failed")

    def advance(self, x_target: float = -1.0, max_steps: int = 0, trace_cap: int = 200000) -> dict:
        trace = np.zeros(trace_cap, dtype=STEP_DTYPE)
        out = OracleOut()
        s = self._lib.oracle_advance(self._h, C.c_double(x_target), C.c_uint32(max_steps), _p(trace), C.c_uint32(trace_cap),
                                     C.byref(out))
        return {"status": s, "trace": trace[:min(out.n_steps, trace_cap)], "seconds": out.seconds, "n_steps": out.n_steps}

    def done(self, x_target: float = -1.0) -> bool:
        return bool(self._lib.oracle_done(self._h, C.c_double(x_target)))

    def finish(self) -> dict:
        labels = np.empty(self.ncells, dtype=np.uint32)
        rc = np.empty(max(self.nrxg, 1), dtype=np.uint32)
        dc = np.empty(self.ndefg, dtype=np.uint32)
        self._lib.oracle_finish(self._h, _p(labels), _p(rc), _p(dc))
        return {"labels": labels, "rxg_counts": rc[: self.nrxg], "defg_counts": dc}

    def time(self) -> float:
        return self._lib.oracle_time(self._h)

    def grainevo(self, nz: int) -> list[dict]:
        """Snapshots of the grain-evolution log taken so far: t, X, step, Sv, counts, area [nz, 2]."""
        out = []
        G = self.ndefg + self.nrxg
        for i in range(self._lib.oracle_log_count(self._h)):
            t, X = C.c_double(), C.c_double()
            st, sv = C.c_uint32(), C.c_uint32()
            cnt = np.empty(G, dtype=np.uint32)
            area = np.empty((nz, 2), dtype=np.uint32)
            self._lib.oracle_log_get(self._h, i, C.byref(t), C.byref(X), C.byref(st), C.byref(sv), _p(cnt), _p(area))
            out.append({"t": t.value, "X": X.value, "step": st.value, "Sv": sv.value, "counts": cnt, "area": area})
        return out

    def binarize(self) -> np.ndarray:
        """1 for recrystallized and infected cells (grid value >= ndefg), as the reference binarizes."""
        b = np.empty(self.ncells, dtype=np.uint8)
        self._lib.oracle_binarize(self._h, _p(b))
        return b

    def close(self) -> None:
        if self._h:
            self._lib.oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class OracleEvo(C.Structure):
    _fields_ = [("ndefg", C.c_uint32), ("nrxg", C.c_uint32), ("nsnap", C.c_uint32), ("t", C.c_void_p), ("counts", C.c_void_p),
                ("final_counts", C.c_void_p), ("tsimend", C.c_double), ("nboxvol", C.c_double), ("grain_class", C.c_void_p)]


def _evos(domains):
    """ctypes descriptors of grain-evolution logs: dicts with ndefg, nrxg, t (snapshots), counts
    [nsnap, G], final [G], tsimend, cells, optionally cls [G]; arrays kept alive with them."""
    keep, arr = [], (OracleEvo * len(domains))()
    for k, d in enumerate(domains):
        t = np.ascontiguousarray(d["t"], dtype=np.float64)
        cnt = np.ascontiguousarray(d["counts"], dtype=np.uint32)
        fin = np.ascontiguousarray(d["final"], dtype=np.uint32)
        cls = None if d.get("cls") is None else np.ascontiguousarray(d["cls"], dtype=np.uint32)
        keep += [t, cnt, fin, cls]
        arr[k] = OracleEvo(d["ndefg"], d["nrxg"], len(t), _p(t), _p(cnt), _p(fin), d["tsimend"], float(d["cells"]), _p(cls))
    return arr, keep


def interp_count(domain: dict, gid: int, when: float) -> float:
    """caHdl::get_interpCellCount restated (SCORE_SolitaryUnitAveraging.cpp:1304-1365)."""
    arr, keep = _evos([domain])
    return _load().oracle_interp_count(arr, gid, when)


def rediscr_kinetics(domains: list, nslots: int):
    """postprocess_rediscr_kinetics restated: (t, rx volume per slot, box volume)."""
    arr, keep = _evos(domains)
    t = np.empty(nslots, dtype=np.float64)
    v = np.empty(nslots, dtype=np.float64)
    box = C.c_double()
    _load().oracle_rediscr_kinetics(arr, len(domains), nslots, _p(t), _p(v), C.byref(box))
    return t, v, box.value


def rediscr_texture(domains: list, nslots: int, nclass: int):
    """postprocess_rediscr_macrotexture restated: (t, volume[nslots, nclass])."""
    arr, keep = _evos(domains)
    t = np.empty(nslots, dtype=np.float64)
    v = np.empty((nslots, nclass), dtype=np.float64)
    _load().oracle_rediscr_macrotexture(arr, len(domains), nslots, nclass, _p(t), _p(v))
    return t, v


def percolation(binarized: np.ndarray, nx: int, ny: int, nz: int, reference_scan: bool = False) -> dict:
    """Clusters of the 1-cells (6-connected, not periodic): the reference's sequential Hoshen-Kopelman
    scan (reference_scan) or the true components; labels in order of first appearance, counts,
    largest, spanning axes and the ascending sizes (SCORE_PercAnalyzer.cpp)."""
    b = np.ascontiguousarray(binarized, dtype=np.uint8).ravel()
    N = nx * ny * nz
    labels = np.empty(N, dtype=np.uint32)
    sizes = np.empty(N // 2 + 2, dtype=np.uint32)
    n, big, perc, spans = C.c_uint32(), C.c_uint32(), C.c_int(), C.c_uint32()
    s = _load().oracle_percolation(_p(b), nx, ny, nz, int(reference_scan), _p(labels), C.byref(n), C.byref(big), C.byref(perc),
                                   C.byref(spans), _p(sizes))
    if s != 0:
        raise MemoryError("oracle_percolation")
    return {"labels": labels, "n_clusters": n.value, "largest": big.value, "percolates": bool(perc.value),
            "spans": spans.value, "sizes": sizes[: n.value].copy()}


def mobility_weight(params, qr, qd) -> float:
    lib = _load()
    a = np.ascontiguousarray(qr, dtype=np.float64)
    b = np.ascontiguousarray(qd, dtype=np.float64)
    return lib.oracle_mobility_weight(C.byref(params), _p(a), _p(b))


def _read_kv(path: Path) -> dict:
    kv = {"rxg": {}, "defg": {}}
    for line in path.read_text().splitlines():
        parts = line.split()
        if len(parts) == 3 and parts[0] in ("rxg", "defg"):
            kv[parts[0]][int(parts[1])] = int(parts[2])
        elif len(parts) == 2:
            kv[parts[0]] = parts[1]
    return kv


def run_ref(mode: str, uds_path, domain, workdir=None, threads: int = 1, timeout: float = 3600) -> dict:
    """Run the reference harness in `mode` (loop | asis | ptab) on `domain`."""
    exe = build_ref()
    if exe is None or not exe.exists():
        raise RuntimeError("reference sources not found: set SCORE_REFERENCE to the SCORE source tree "
                           "(no prebuilt harness in oracle/_ref/ either)")
    wd = Path(workdir or tempfile.mkdtemp(prefix="scoreref_"))
    wd.mkdir(parents=True, exist_ok=True)
    scdm = domain.write_scdm(wd / "domain.scdm")
    prefix = wd / "out"
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    r = subprocess.run([str(exe), mode, str(uds_path), str(scdm), str(prefix)], cwd=wd, env=env, capture_output=True,
                       text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"reference harness failed ({r.returncode}): {r.stderr[-2000:]}")
    res = {"workdir": wd}
    if mode == "ptab":
        n = domain.nrxg * domain.ndefg
        res["ptab"] = np.fromfile(f"{prefix}.ptab", dtype=np.float64, count=n).reshape(domain.nrxg, domain.ndefg)
        res["ptabnuc"] = np.fromfile(f"{prefix}.ptabnuc", dtype=np.float64, count=n).reshape(domain.nrxg, domain.ndefg)
    elif mode == "asis":
        res.update(_read_kv(Path(f"{prefix}.asis")))
    else:
        res.update(_read_kv(Path(f"{prefix}.summary")))
        res["trace"] = np.fromfile(f"{prefix}.trace", dtype=REF_STEP_DTYPE)
        res["labels"] = np.fromfile(f"{prefix}.labels", dtype=np.uint32)
    return res
