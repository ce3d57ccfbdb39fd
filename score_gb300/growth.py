"""Host-side API of the GB300 growth step, mirroring SCORE's growth machine.

The reference drives one domain through
``solve_INITIALIZATION -> ... -> solve_REPLACE_CA_STRUCTURE -> solve_RXGROWTH``
(src/SCORE_Kernel.cpp:1693-1756); :class:`GrowthMachine` exposes the same
sequence over the C ABI: ``load_domain`` (structure + nuclei pools),
``place_nuclei`` (site-saturated nucleation), ``step`` / ``run_until`` (the
growth loop) and ``labels`` (final grain ids by the clarify rule).  Every call
runs the CUDA path; there is no CPU fallback — without a GPU the constructor
raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _abi
from ._abi import GenParams, GrainEvoInfo, Params, Percolation, ScoreError, StepStats, Timing, Tune


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def lib():
    return _abi.load()


def host_lib():
    """The host-only library: parameters, host weights and the generator never need CUDA."""
    return _abi.load_host()


# ---------------------------------------------------------------- parameters
def default_params() -> Params:
    p = Params()
    host_lib().score_params_default(C.byref(p))
    return p


def read_uds(path: str | Path) -> Params:
    """Parse a SCORE .uds input file (ensembleHdl::init_parameter semantics)."""
    p = Params()
    s = host_lib().score_uds_read(str(path).encode(), C.byref(p))
    if s != _abi.OK:
        raise ScoreError(s, f"cannot read {path}")
    return p


@dataclass
class UdsSpec:
    """The growth-relevant keywords of a SCORE .uds input file.

    Values are written as text exactly as given, so the reference's parser and
    this library's parser read identical doubles (table columns become floats,
    temperatures are Celsius, activation enthalpies eV — as in the reference).
    """
    nx: int = 128
    ny: int = 128
    nz: int = 128
    cellsize_um: str = "1.0"
    xmax: str = "0.99"
    tmax: str = "360000.0"
    nmax: str = "1000000"
    maxfill: str = "0.1"
    initial_cache: str = "0.10"
    recache: str = "1.0"
    defragmentation: int = 0
    defrag_x: list = field(default_factory=lambda: ["0.5"])
    logpoints: list = field(default_factory=lambda: ["1.0"])   # SingleGrainVolOverTime: X of the grain-evolution log
    area_threshold: int = 13                                   # RX area profile: smallest rx grain section counted
    G0: str = "85.0e9"
    bZeroCelsius: str = "248.5e-12"
    mobility_model: int = 1
    LAGBm0: str = "300.0"
    LAGBHact: str = "2.45"
    HAGBm0: str = "300.0"
    HAGBHact: str = "2.45"
    GSm0: str = "300.0"
    GSHact: str = "2.45"
    RH_HAGBm0: str = "300.0"
    RH_HAGBHact: str = "2.45"
    RH_cut: str = "0.9"
    RH_trans: str = "5.0"
    RH_exponent: str = "9.0"
    recovery: int = 0
    recovery_k: str = "0.01"
    zener: int = 0
    zener_table: list = field(default_factory=lambda: [("0.0", "1.0e6"), ("360000.0", "1.0e6")])
    schedule: list = field(default_factory=lambda: [("0.0", "726.85"), ("360000.0", "726.85")])
    boundary: int = 0
    precision: int = 0
    border_policy: int = 0

    def text(self) -> str:
        L = []
        a = L.append
        a("|| RuntimeControl || *(ss) || Parameter, Value")
        for k, v in [("XMAX", self.xmax), ("TIMEMAX", self.tmax), ("NMAX", self.nmax), ("PERCOLATIONANALYSIS", "0"),
                     ("MAXFILLPERSTEP", self.maxfill), ("RediscretizationSteps", "1000"),
                     ("InitialCacheSizeRXCells", self.initial_cache), ("ReCacheSizeRXCells", self.recache),
                     ("OnTheFlyDefragmentation", str(self.defragmentation)), ("SolitaryUnitPostProcessing", "0"),
                     ("ReadEBSDMapping", "0"), ("ReadEBSDStepsize", "0.25E-06")]:
            a(f'"{k}"\t"{v}"')
        a("")
        a("|| SimulationOutput || *(ss) || Parameter, Value")
        for k, v in [("RenderingOfMicrostructure", "0"), ("RenderingColorModel", "1"), ("RenderingFileFormat", "1"),
                     ("RenderingBoundaries", "0"), ("OutputLogBoundaries", "0"), ("OutputRXFrontStats", "0"),
                     ("OutputThreadProfiling", "1"), ("OutputSingleGrainStats", "0"), ("OutputDAMASKGeometryFile", "0"),
                     ("OutputArtificialSEMEBSD", "0")]:
            a(f'"{k}"\t"{v}"')
        a("")
        a("|| EnsembleDefinition || *(ss) || Parameter, Value")
        for k, v in [("CAEnsembleSize", "1"), ("CellSize", self.cellsize_um), ("3DCAEdgeLengthInCellsRD", str(self.nx)),
                     ("3DCAEdgeLengthInCellsTD", str(self.ny)), ("3DCAEdgeLengthInCellsND", str(self.nz)),
                     ("MeanDefGrainSizeinRD", "30.0"), ("MeanDefGrainSizeinTD", "30.0"), ("MeanDefGrainSizeinND", "30.0"),
                     ("DefStructureSynthesis", "1"), ("MeanDefSizePoissonDiameter", "30.0")]:
            a(f'"{k}"\t"{v}"')
        a("")
        a("|| NucleationModeling || *(ss) || Parameter, Value")
        for k, v in [("NucleationDensityLocalCSR", "1"), ("CSRNucleation", "1"), ("ClusteredNucleation", "0"),
                     ("ClusteredNucleationNCluster", "1"), ("ClusteredNucleationLCluster", "1.0"),
                     ("ClusteredNucleationScaling", "1.0"), ("ClusteredNucleationExtendA", "1"),
                     ("ClusteredNucleationExtendB", "1"), ("ClusteredNucleationExtendC", "1"), ("GBNucleation", "0"),
                     ("GBNucDensity2Number", "1.0E-4"), ("GBNucRhoDiff2Density", "5E-14"), ("GBNucMaximumScatter", "5.0"),
                     ("IncubationTimeModel", "1"), ("IncubationTimeScatter", "1000.0")]:
            a(f'"{k}"\t"{v}"')
        a("")
        a("|| MaterialProperties || *(ss) || Parameter, Value")
        for k, v in [("ZeroKelvinShearModulusG0", self.G0), ("FirstOrderdG0dT", "0.0"), ("ZeroCelsiusBurgersVector", self.bZeroCelsius),
                     ("AlloyConstantThermalExpCoeff", "1.0"), ("FirstOrderThermalExpCoeff", "0.0"),
                     ("SecondOrderThermalExpCoeff", "0.0"), ("MeltingTemperature", "800.0")]:
            a(f'"{k}"\t"{v}"')
        a("")
        a("|| BoundaryMobilityModel || *(ss) || Parameter, Value")
        for k, v in [("MobilityModel", str(self.mobility_model)), ("LAGBm0", self.LAGBm0), ("LAGBHact", self.LAGBHact),
                     ("HAGBm0", self.HAGBm0), ("HAGBHact", self.HAGBHact), ("GSm0", self.GSm0), ("GSHact", self.GSHact),
                     ("RHModelHAGBm0", self.RH_HAGBm0), ("RHModelHAGBHact", self.RH_HAGBHact),
                     ("RHModelLAGBHAGBCut", self.RH_cut), ("RHModelLAGBHAGBTrans", self.RH_trans),
                     ("RHModelLAGBHAGBExponent", self.RH_exponent)]:
            a(f'"{k}"\t"{v}"')
        a("")
        a("|| RecoveryParameter || *(ss) || Parameter, Value")
        for k, v in [("RecoveryConsider", str(self.recovery)), ("RecoveryVacancyDiffGeometry", "1.0"),
                     ("RecoveryVacancyDiffPreexp", "1.0"), ("RecoveryVacancyDiffHact", "2.9"),
                     ("RecoverySoluteDiffPreexp", "1.0"), ("RecoverySoluteDiffHact", "1.6"),
                     ("RecoverySoluteLsPropFactor", "1.0"), ("RecoverySoluteConcentration", "1.0"),
                     ("RecoveryParameterAlpha3", "1.0"), ("RecoveryParameterKappa2", "0.1"), ("RecoveryParameterC3", "1.0"),
                     ("RecoveryParameterC4", "1.0"), ("RecoveryParameterC5", "0.65"), ("RecoveryHyperbolicK", self.recovery_k)]:
            a(f'"{k}"\t"{v}"')
        a("")
        a("|| DragParameter || *(ss) || Parameter, Value")
        for k, v in [("ZenerConsider", str(self.zener)), ("ZenerAlpha", "1.5"), ("ZenerGamma", "0.324")]:
            a(f'"{k}"\t"{v}"')
        a("")
        a("|| EvoMicrochemistry || *(ff) || time, fr")
        for t, fr in self.zener_table:
            a(f"{t}\t{fr}")
        a("")
        a("|| IdealComponents || *(sffff) || Name, Bunge1, Bunge2, Bunge3, scatter")
        a('"Cube"\t0.0\t0.0\t0.0\t10.0')
        a("")
        a("|| AnnealingSchedule || *(ff) || time, temperature")
        for t, T in self.schedule:
            a(f"{t}\t{T}")
        a("")
        a("|| DeformedGrainsPool || *(ffff) || Bunge1, Bunge2, Bunge3, rho")
        a("10.0\t20.0\t30.0\t1.0e15")
        a("")
        a("|| RXGrainsPool || *(ffff) || Bunge1, Bunge2, Bunge3, tincub")
        a("40.0\t50.0\t60.0\t0.0")
        a("")
        a("|| HeuristicRXFrontListDefragmentation || *(sf) || Name, X")
        for i, x in enumerate(self.defrag_x):
            a(f'"D{i}"\t{x}')
        a("")
        a("|| SingleGrainVolOverTime || *(sf) || Name, X")
        for i, x in enumerate(self.logpoints):
            a(f'"L{i}"\t{x}')
        a("")
        a("|| GB300Options || *(ss) || Parameter, Value")
        for k, v in [("Boundary", str(self.boundary)), ("Precision", str(self.precision)), ("BorderPolicy", str(self.border_policy)),
                     ("RXAreaThreshold", str(self.area_threshold))]:
            a(f'"{k}"\t"{v}"')
        a("")
        return "\n".join(L) + "\n"

    def write(self, path: str | Path) -> Path:
        path = Path(path)
        path.write_text(self.text())
        return path


# ---------------------------------------------------------------- domains
@dataclass
class Domain:
    """One solitary-unit domain: deformed-grain label grid plus both grain pools."""
    nx: int
    ny: int
    nz: int
    grid: np.ndarray          # uint32[nz, ny, nx] (x fastest), deformed ids
    defg_quat: np.ndarray     # float64[ndefg, 4]
    defg_rho0: np.ndarray     # float64[ndefg]
    rxg_quat: np.ndarray      # float64[nrxg, 4]
    rxg_site: np.ndarray      # uint32[nrxg] linear sites
    rxg_tincub: np.ndarray    # float64[nrxg]

    @property
    def ncells(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def ndefg(self) -> int:
        return int(self.defg_rho0.shape[0])

    @property
    def nrxg(self) -> int:
        return int(self.rxg_site.shape[0])

    def write_scdm(self, path: str | Path) -> Path:
        """Binary domain file read by the reference harness (magic SCDM, version 1)."""
        path = Path(path)
        with open(path, "wb") as f:
            f.write(b"SCDM")
            f.write(np.array([1, self.nx, self.ny, self.nz, self.ndefg, self.nrxg], dtype=np.uint32).tobytes())
            f.write(np.ascontiguousarray(self.grid, dtype=np.uint32).tobytes())
            d = np.concatenate([self.defg_quat, self.defg_rho0[:, None]], axis=1)
            f.write(np.ascontiguousarray(d, dtype=np.float64).tobytes())
            f.write(np.ascontiguousarray(self.rxg_quat, dtype=np.float64).tobytes())
            f.write(np.ascontiguousarray(self.rxg_site, dtype=np.uint32).tobytes())
            f.write(np.ascontiguousarray(self.rxg_tincub, dtype=np.float64).tobytes())
        return path


def generate_domain(nx: int, ny: int, nz: int, ngrains: int, nnuclei: int, seed: int = 0, device: int | None = None,
                    **kw) -> Domain:
    """Deterministic synthetic domain (identical bits on x86-64 and aarch64 hosts).

    Keyword overrides map onto score_gen_params: rho_mean, rho_sigma, rho_mode,
    rho_lo, rho_hi, aspect (3-tuple), ori_mode, ncomp, scatter_deg, site_mode,
    gb_fraction, nucleation_rate.  With `device` the Voronoi label fill runs on that
    GPU (score_generate_domain_gpu): the same bits, the CUDA library instead of the
    host-only one.
    """
    g = GenParams()
    host_lib().score_gen_default(C.byref(g))
    g.nx, g.ny, g.nz, g.ngrains, g.nnuclei, g.seed = nx, ny, nz, ngrains, nnuclei, seed
    for k, v in kw.items():
        if k == "aspect":
            for i in range(3):
                g.aspect[i] = float(v[i])
        else:
            setattr(g, k, v)
    grid = np.empty((nz, ny, nx), dtype=np.uint32)
    dq = np.empty((ngrains, 4), dtype=np.float64)
    rho = np.empty(ngrains, dtype=np.float64)
    rq = np.empty((nnuclei, 4), dtype=np.float64)
    site = np.empty(nnuclei, dtype=np.uint32)
    tinc = np.empty(nnuclei, dtype=np.float64)
    if device is None:
        s = host_lib().score_generate_domain(C.byref(g), _ptr(grid), _ptr(dq), _ptr(rho), _ptr(rq), _ptr(site), _ptr(tinc))
    else:
        s = lib().score_generate_domain_gpu(C.byref(g), _ptr(grid), _ptr(dq), _ptr(rho), _ptr(rq), _ptr(site), _ptr(tinc), device)
    if s != _abi.OK:
        raise ScoreError(s, "domain generation failed")
    return Domain(nx, ny, nz, grid, dq, rho, rq, site, tinc)


def mobility_weight(params: Params, q_rx, q_def) -> float:
    """Host FP64 P(rxg, defg), the reference's formula (SCORE_Kernel.cpp:2460-2527)."""
    out = C.c_double()
    qr = np.ascontiguousarray(q_rx, dtype=np.float64)
    qd = np.ascontiguousarray(q_def, dtype=np.float64)
    lib().score_mobility_weight(C.byref(params), _ptr(qr), _ptr(qd), C.byref(out))
    return out.value


def stats_dict(s: StepStats) -> dict:
    return {k: (list(getattr(s, k)) if k in ("next_never", "n_recycled") else getattr(s, k)) for k, _ in StepStats._fields_}


def _percolation(d: Domain, call, connected: bool, labels: bool) -> dict:
    r = Percolation()
    sizes = np.empty(d.ncells // 2 + 2, dtype=np.uint32)
    lab = np.empty((d.nz, d.ny, d.nx), dtype=np.uint32) if labels else None
    call(1 if connected else 0, C.byref(r), _ptr(sizes), sizes.size, _ptr(lab))
    out = {"n_clusters": r.n_clusters, "largest": r.largest, "PL": r.PL, "percolates": bool(r.percolates), "spans": r.spans,
           "sizes": sizes[: r.n_clusters].copy()}
    if labels:
        out["labels"] = lab
    return out


# ---------------------------------------------------------------- growth machine
class GrowthMachine:
    """One domain on one GPU (caHdl + its region fronts, SCORE_Kernel.h:1008-1584)."""

    def __init__(self, params: Params, device: int = 0):
        self._lib = lib()
        self._ctx = C.c_void_p()
        self.params = params
        s = self._lib.score_create(C.byref(self._ctx), C.byref(params), device)
        if s != _abi.OK:
            raise ScoreError(s, self._lib.score_status_string(s).decode())
        self.domain: Domain | None = None

    def _check(self, s: int) -> None:
        if s != _abi.OK:
            msg = self._lib.score_last_error(self._ctx).decode() if self._ctx else ""
            raise ScoreError(s, msg or self._lib.score_status_string(s).decode())

    def load_domain(self, d: Domain, ptable: np.ndarray | None = None) -> None:
        self.domain = d
        self._keep = [np.ascontiguousarray(x) for x in (d.grid, d.defg_quat, d.defg_rho0, d.rxg_quat, d.rxg_site, d.rxg_tincub)]
        if ptable is not None:
            ptable = np.ascontiguousarray(ptable, dtype=np.float64)
            self._keep.append(ptable)
        g, dq, rho, rq, site, tinc = self._keep[:6]
        self._check(self._lib.score_load_domain(self._ctx, _ptr(g), _ptr(dq), _ptr(rho), d.ndefg, _ptr(rq), _ptr(site),
                                                _ptr(tinc), d.nrxg, _ptr(ptable)))

    def restart(self) -> None:
        """Back to the just-loaded state from device-resident inputs (no host copy)."""
        self._check(self._lib.score_restart(self._ctx))

    def place_nuclei(self) -> int:
        n = C.c_uint32()
        self._check(self._lib.score_place_nuclei(self._ctx, C.byref(n)))
        return n.value

    def step(self) -> StepStats:
        st = StepStats()
        self._check(self._lib.score_step(self._ctx, C.byref(st)))
        return st

    def run_until(self, x_target: float = -1.0, max_trace: int = 100000) -> list[StepStats]:
        trace = (StepStats * max_trace)()
        n = C.c_uint32()
        self._check(self._lib.score_run_until(self._ctx, x_target, trace, max_trace, C.byref(n)))
        return list(trace[: min(n.value, max_trace)])

    def solve_rxgrowth(self, x_target: float = -1.0) -> list[StepStats]:
        """Nucleation followed by the full step loop (caHdl::solve_RXGROWTH)."""
        self.place_nuclei()
        return self.run_until(x_target)

    def stats(self) -> StepStats:
        st = StepStats()
        self._check(self._lib.score_get_stats(self._ctx, C.byref(st)))
        return st

    def labels(self, out: np.ndarray | None = None) -> np.ndarray:
        d = self.domain
        if out is None:
            out = np.empty((d.nz, d.ny, d.nx), dtype=np.uint32)
        self._check(self._lib.score_export_labels(self._ctx, _ptr(out)))
        return out

    def grain_counts(self) -> tuple[np.ndarray, np.ndarray]:
        d = self.domain
        r = np.empty(d.nrxg, dtype=np.uint32)
        g = np.empty(d.ndefg, dtype=np.uint32)
        self._check(self._lib.score_grain_counts(self._ctx, _ptr(r), _ptr(g)))
        return r, g

    def timing(self) -> Timing:
        t = Timing()
        self._check(self._lib.score_get_timing(self._ctx, C.byref(t)))
        return t

    def grainevo(self) -> list[tuple[GrainEvoInfo, np.ndarray, np.ndarray]]:
        """The last run's grain-evolution log (log_grainevo + log_rxareaprofile at the
        SingleGrainVolOverTime logpoints): per snapshot (info, counts[ndefg + nrxg],
        rx area profile [nz, 2])."""
        d = self.domain
        n = C.c_uint32()
        self._check(self._lib.score_grainevo_count(self._ctx, C.byref(n)))
        out = []
        for i in range(n.value):
            info = GrainEvoInfo()
            cnt = np.empty(d.ndefg + d.nrxg, dtype=np.uint32)
            area = np.empty((d.nz, 2), dtype=np.uint32)
            self._check(self._lib.score_grainevo(self._ctx, i, C.byref(info), _ptr(cnt), _ptr(area)))
            out.append((info, cnt, area))
        return out

    def percolation(self, connected: bool = False, labels: bool = False) -> dict:
        """Clusters of the recrystallized and infected cells now (log_PERCOLATION): the reference's
        clusters, or the true 6-connected ones; count, largest, P_L, percolates, spans, sorted sizes,
        optionally every cell's label."""
        return _percolation(self.domain, lambda *a: self._check(self._lib.score_percolation_analyze(self._ctx, *a)), connected, labels)

    def rediscr_kinetics(self, nslots: int) -> tuple[np.ndarray, np.ndarray, float]:
        """X(t) of this domain on nslots rediscretized times: (t, rx volume, box volume)."""
        t = np.empty(nslots, dtype=np.float64)
        v = np.empty(nslots, dtype=np.float64)
        box = C.c_double()
        self._check(self._lib.score_rediscr_kinetics(self._ctx, nslots, _ptr(t), _ptr(v), C.byref(box)))
        return t, v, box.value

    def tune(self) -> Tune:
        t = Tune()
        self._check(self._lib.score_get_tune(self._ctx, C.byref(t)))
        return t

    def set_tune(self, t: Tune | None = None, **kw) -> None:
        """Launch configuration (items, *_blocks_per_sm, use_graph); results never depend on it."""
        t = t or self.tune()
        for k, v in kw.items():
            setattr(t, k, v)
        self._check(self._lib.score_set_tune(self._ctx, C.byref(t)))

    def autotune(self, x_target: float = -1.0, max_steps: int = 0) -> Tune:
        """Pick the fastest launch configuration on real steps; leaves the domain restarted
        with its nuclei placed."""
        t = Tune()
        self._check(self._lib.score_autotune(self._ctx, x_target, max_steps, C.byref(t)))
        return t

    def close(self) -> None:
        if self._ctx:
            self._lib.score_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- batched ensemble
class Batch:
    """Many independent domains stepped together in one sequence of launches per step
    (the reference's ensemble of solitary units, SCORE_Kernel.cpp:1640-1756)."""

    def __init__(self, params: list[Params], device: int = 0):
        self._lib = lib()
        self._b = C.c_void_p()
        arr = (Params * len(params))(*params)
        s = self._lib.score_batch_create(C.byref(self._b), arr, len(params), device)
        if s != _abi.OK:
            raise ScoreError(s, self._lib.score_status_string(s).decode())
        self.params = list(params)
        self.domains: list[Domain | None] = [None] * len(params)
        self._keep: dict[int, list] = {}

    def __len__(self) -> int:
        return len(self.params)

    def _check(self, s: int) -> None:
        if s != _abi.OK:
            msg = self._lib.score_batch_last_error(self._b).decode() if self._b else ""
            raise ScoreError(s, msg or self._lib.score_status_string(s).decode())

    def load_domain(self, i: int, d: Domain, ptable: np.ndarray | None = None) -> None:
        keep = [np.ascontiguousarray(x) for x in (d.grid, d.defg_quat, d.defg_rho0, d.rxg_quat, d.rxg_site, d.rxg_tincub)]
        if ptable is not None:
            keep.append(np.ascontiguousarray(ptable, dtype=np.float64))
        g, dq, rho, rq, site, tinc = keep[:6]
        self._check(self._lib.score_batch_load_domain(self._b, i, _ptr(g), _ptr(dq), _ptr(rho), d.ndefg, _ptr(rq), _ptr(site),
                                                      _ptr(tinc), d.nrxg, _ptr(keep[6] if ptable is not None else None)))
        self._keep[i] = keep
        self.domains[i] = d

    def restart(self) -> None:
        self._check(self._lib.score_batch_restart(self._b))

    def place_nuclei(self) -> None:
        self._check(self._lib.score_batch_place_nuclei(self._b))

    def run_until(self, x_target: float = -1.0, max_steps: int = 0) -> int:
        n = C.c_uint32()
        self._check(self._lib.score_batch_run_until(self._b, x_target, max_steps, C.byref(n)))
        return n.value

    def trace(self, i: int) -> list[StepStats]:
        n = C.c_uint32()
        self._check(self._lib.score_batch_trace(self._b, i, None, 0, C.byref(n)))
        buf = (StepStats * max(1, n.value))()
        self._check(self._lib.score_batch_trace(self._b, i, buf, n.value, C.byref(n)))
        return list(buf[: n.value])

    def stats(self, i: int) -> StepStats:
        st = StepStats()
        self._check(self._lib.score_batch_get_stats(self._b, i, C.byref(st)))
        return st

    def labels(self, i: int, out: np.ndarray | None = None) -> np.ndarray:
        d = self.domains[i]
        if out is None:
            out = np.empty((d.nz, d.ny, d.nx), dtype=np.uint32)
        self._check(self._lib.score_batch_export_labels(self._b, i, _ptr(out)))
        return out

    def grain_counts(self, i: int) -> tuple[np.ndarray, np.ndarray]:
        d = self.domains[i]
        r = np.empty(d.nrxg, dtype=np.uint32)
        g = np.empty(d.ndefg, dtype=np.uint32)
        self._check(self._lib.score_batch_grain_counts(self._b, i, _ptr(r), _ptr(g)))
        return r, g

    def timing(self) -> Timing:
        t = Timing()
        self._check(self._lib.score_batch_get_timing(self._b, C.byref(t)))
        return t

    def grainevo(self, i: int) -> list[tuple[GrainEvoInfo, np.ndarray, np.ndarray]]:
        """Domain i's grain-evolution log of the last run (see GrowthMachine.grainevo)."""
        d = self.domains[i]
        n = C.c_uint32()
        self._check(self._lib.score_batch_grainevo_count(self._b, i, C.byref(n)))
        out = []
        for k in range(n.value):
            info = GrainEvoInfo()
            cnt = np.empty(d.ndefg + d.nrxg, dtype=np.uint32)
            area = np.empty((d.nz, 2), dtype=np.uint32)
            self._check(self._lib.score_batch_grainevo(self._b, i, k, C.byref(info), _ptr(cnt), _ptr(area)))
            out.append((info, cnt, area))
        return out

    def rediscr_kinetics(self, nslots: int) -> tuple[np.ndarray, np.ndarray, float]:
        """Ensemble recrystallization kinetics on nslots rediscretized times, on the device
        (postprocess_rediscr_kinetics): (t, rx volume, box volume); X = rx volume / box volume."""
        t = np.empty(nslots, dtype=np.float64)
        v = np.empty(nslots, dtype=np.float64)
        box = C.c_double()
        self._check(self._lib.score_batch_rediscr_kinetics(self._b, nslots, _ptr(t), _ptr(v), C.byref(box)))
        return t, v, box.value

    def rediscr_texture(self, nslots: int, grain_class: np.ndarray, nclass: int) -> tuple[np.ndarray, np.ndarray]:
        """Ensemble volume per orientation class on nslots rediscretized times, on the device
        (postprocess_rediscr_macrotexture); grain_class: every domain's ndefg + nrxg classes in
        domain order.  Returns (t, volume[nslots, nclass])."""
        cls = np.ascontiguousarray(grain_class, dtype=np.uint32)
        t = np.empty(nslots, dtype=np.float64)
        v = np.empty((nslots, nclass), dtype=np.float64)
        self._check(self._lib.score_batch_rediscr_texture(self._b, nslots, _ptr(cls), nclass, _ptr(t), _ptr(v)))
        return t, v

    def percolation(self, i: int, connected: bool = False, labels: bool = False) -> dict:
        """Domain i's clusters now (see GrowthMachine.percolation)."""
        return _percolation(self.domains[i], lambda *a: self._check(self._lib.score_batch_percolation_analyze(self._b, i, *a)), connected,
                            labels)

    def final_grain_sizes(self) -> np.ndarray:
        """Every domain's rx grains' final cell counts, in domain order."""
        n = sum(d.nrxg for d in self.domains)
        out = np.empty(n, dtype=np.uint32)
        self._check(self._lib.score_batch_final_grain_sizes(self._b, _ptr(out)))
        return out

    def tune(self) -> Tune:
        t = Tune()
        self._check(self._lib.score_batch_get_tune(self._b, C.byref(t)))
        return t

    def set_tune(self, t: Tune | None = None, **kw) -> None:
        t = t or self.tune()
        for k, v in kw.items():
            setattr(t, k, v)
        self._check(self._lib.score_batch_set_tune(self._b, C.byref(t)))

    def autotune(self, x_target: float = -1.0, max_steps: int = 0) -> Tune:
        """Fastest launch configuration on real steps; leaves the batch restarted with its
        nuclei placed."""
        t = Tune()
        self._check(self._lib.score_batch_autotune(self._b, x_target, max_steps, C.byref(t)))
        return t

    def close(self) -> None:
        if self._b:
            self._lib.score_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
