"""ctypes binding of include/score_gb300.h (the C ABI of the growth step).

Struct layouts here must match the header field for field; tests check the
sizes against the library's own view of them.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

MAX_TABLE = 256

OK = 0
ERR_ARG = -1
ERR_CUDA = -2
ERR_NOMEM = -3
ERR_CAPACITY = -4
ERR_BORDER_CAPACITY = -5
ERR_TIMEOUT = -6
ERR_STATE = -7
ERR_IO = -8
ERR_KEYLIMIT = -9
ERR_NOT_BUILT = -10
ERR_SCRATCH_LIMIT = -11

MOBILITY_SEBALD_GOTTSTEIN = 1
MOBILITY_ROLLETT_HOLM = 2
RECOVERY_NONE, RECOVERY_NES_VACCOREDIFF, RECOVERY_NES_SOLUTEDRAG, RECOVERY_MICHALAKPAXTON = 0, 1, 2, 3
RECOVERY_HYPERBOLIC = 10
ZENER_NONE, ZENER_CONSTANT, ZENER_TIMEDEP = 0, 1, 2
BOUNDARY_REFERENCE, BOUNDARY_PERIODIC = 0, 1
PRECISION_FP64, PRECISION_FP32_KAHAN = 0, 1
BORDER_REFERENCE_LIMIT, BORDER_GROW = 0, 1

_d = C.c_double
_u32 = C.c_uint32
_i32 = C.c_int32


class Params(C.Structure):
    _fields_ = [
        ("nx", _u32), ("ny", _u32), ("nz", _u32),
        ("cellsize", _d), ("xmax", _d), ("tmax", _d), ("nmax", _u32),
        ("maxfillperstep", _d), ("initial_cache", _d), ("recache", _d),
        ("defragmentation", _i32), ("n_defrag", _u32), ("defrag_x", _d * MAX_TABLE),
        ("G0", _d), ("dGdt", _d), ("bZeroCelsius", _d), ("Tmelt", _d),
        ("mobility_model", _i32),
        ("LAGBm0", _d), ("LAGBHact", _d), ("HAGBm0", _d), ("HAGBHact", _d), ("GSm0", _d), ("GSHact", _d),
        ("RH_HAGBm0", _d), ("RH_HAGBHact", _d), ("RH_cut", _d), ("RH_trans", _d), ("RH_exponent", _d),
        ("recovery_model", _i32),
        ("VacancyDiffD0", _d), ("VacancyDiffHact", _d), ("SoluteDiffD0", _d), ("SoluteDiffHact", _d),
        ("SoluteLsPropFactor", _d), ("SoluteConcentration", _d),
        ("NesAlpha3", _d), ("NesKappa2", _d), ("NesC3", _d), ("NesC4", _d), ("NesC5", _d),
        ("recovery_k", _d),
        ("zener_model", _i32), ("zener_alpha", _d), ("zener_gamma", _d),
        ("n_zener", _u32), ("zener_time", _d * MAX_TABLE), ("zener_fr", _d * MAX_TABLE),
        ("n_schedule", _u32), ("sched_time", _d * MAX_TABLE), ("sched_temp", _d * MAX_TABLE),
        ("boundary", _i32), ("precision", _i32), ("border_policy", _i32), ("reserved", _i32),
        ("n_logpoints", _u32), ("logpoint_x", _d * MAX_TABLE), ("rxarea_threshold", _u32), ("reserved2", _u32),
    ]


class StepStats(C.Structure):
    _fields_ = [
        ("step", _u32), ("n_nuclei", _u32), ("t", _d), ("dt", _d), ("dt_used", _d),
        ("Xcells", _d), ("X", _d), ("Sv", C.c_uint64), ("n_full", C.c_uint64), ("n_new", C.c_uint64),
        ("Pmax", _d), ("rhomax", _d), ("dXstep", _d),
        ("next_never", _u32 * 2), ("n_recycled", _u32 * 2), ("p_misses", _u32), ("reserved", _u32),
    ]


class GrainEvoInfo(C.Structure):
    _fields_ = [("t", _d), ("X", _d), ("step", _u32), ("Sv", _u32)]


class Percolation(C.Structure):
    _fields_ = [("n_clusters", _u32), ("largest", _u32), ("PL", _d), ("percolates", _i32), ("spans", _u32)]


class Timing(C.Structure):
    _fields_ = [
        ("total_ms", _d), ("grow_ms", _d), ("claim_ms", _d), ("commit_ms", _d), ("host_ms", _d),
        ("grow_launches", C.c_uint64), ("grow_bytes", _d), ("step_bytes", _d), ("kernel_launches", C.c_uint64),
        ("run_ms", _d), ("fill_ms", _d), ("wait_ms", _d), ("weights_ms", _d), ("pre_ms", _d), ("post_ms", _d),
        ("timed_steps", C.c_uint64),
    ]


class Tune(C.Structure):
    _fields_ = [
        ("items", _i32), ("fill_blocks_per_sm", _i32), ("claim_blocks_per_sm", _i32), ("commit_blocks_per_sm", _i32),
        ("use_graph", _i32), ("spec_holes_pct", _i32), ("timing_every", _i32), ("steps", _u32), ("fill_ns_per_slot", _d), ("claim_ns_per_cell", _d),
        ("commit_ns_per_cell", _d),
    ]


class GenParams(C.Structure):
    _fields_ = [
        ("nx", _u32), ("ny", _u32), ("nz", _u32), ("ngrains", _u32), ("nnuclei", _u32),
        ("seed", C.c_uint64), ("rho_mean", _d), ("rho_sigma", _d), ("rho_mode", _i32),
        ("rho_lo", _d), ("rho_hi", _d), ("aspect", _d * 3), ("ori_mode", _i32), ("ncomp", _u32),
        ("scatter_deg", _d), ("site_mode", _i32), ("gb_fraction", _d), ("nucleation_rate", _d),
    ]


_P = C.POINTER
_vp = C.c_void_p

# name -> (restype, argtypes); every symbol the header declares
SIGNATURES = {
    "score_abi_version": (C.c_int, []),
    "score_status_string": (C.c_char_p, [C.c_int]),
    "score_params_default": (C.c_int, [_P(Params)]),
    "score_uds_read": (C.c_int, [C.c_char_p, _P(Params)]),
    "score_create": (C.c_int, [_P(_vp), _P(Params), C.c_int]),
    "score_destroy": (None, [_vp]),
    "score_last_error": (C.c_char_p, [_vp]),
    "score_load_domain": (C.c_int, [_vp, _vp, _vp, _vp, _u32, _vp, _vp, _vp, _u32, _vp]),
    "score_restart": (C.c_int, [_vp]),
    "score_place_nuclei": (C.c_int, [_vp, _P(_u32)]),
    "score_step": (C.c_int, [_vp, _P(StepStats)]),
    "score_run_until": (C.c_int, [_vp, _d, _P(StepStats), _u32, _P(_u32)]),
    "score_get_stats": (C.c_int, [_vp, _P(StepStats)]),
    "score_export_labels": (C.c_int, [_vp, _vp]),
    "score_grain_counts": (C.c_int, [_vp, _vp, _vp]),
    "score_get_timing": (C.c_int, [_vp, _P(Timing)]),
    "score_get_tune": (C.c_int, [_vp, _P(Tune)]),
    "score_set_tune": (C.c_int, [_vp, _P(Tune)]),
    "score_autotune": (C.c_int, [_vp, _d, _u32, _P(Tune)]),
    "score_batch_create": (C.c_int, [_P(_vp), _P(Params), _u32, C.c_int]),
    "score_batch_destroy": (None, [_vp]),
    "score_batch_last_error": (C.c_char_p, [_vp]),
    "score_batch_load_domain": (C.c_int, [_vp, _u32, _vp, _vp, _vp, _u32, _vp, _vp, _vp, _u32, _vp]),
    "score_batch_restart": (C.c_int, [_vp]),
    "score_batch_place_nuclei": (C.c_int, [_vp]),
    "score_batch_run_until": (C.c_int, [_vp, _d, _u32, _P(_u32)]),
    "score_batch_get_stats": (C.c_int, [_vp, _u32, _P(StepStats)]),
    "score_batch_trace": (C.c_int, [_vp, _u32, _P(StepStats), _u32, _P(_u32)]),
    "score_batch_export_labels": (C.c_int, [_vp, _u32, _vp]),
    "score_batch_grain_counts": (C.c_int, [_vp, _u32, _vp, _vp]),
    "score_batch_get_timing": (C.c_int, [_vp, _P(Timing)]),
    "score_batch_get_tune": (C.c_int, [_vp, _P(Tune)]),
    "score_batch_set_tune": (C.c_int, [_vp, _P(Tune)]),
    "score_batch_autotune": (C.c_int, [_vp, _d, _u32, _P(Tune)]),
    "score_grainevo_count": (C.c_int, [_vp, _P(_u32)]),
    "score_grainevo": (C.c_int, [_vp, _u32, _P(GrainEvoInfo), _vp, _vp]),
    "score_batch_grainevo_count": (C.c_int, [_vp, _u32, _P(_u32)]),
    "score_batch_grainevo": (C.c_int, [_vp, _u32, _u32, _P(GrainEvoInfo), _vp, _vp]),
    "score_rediscr_kinetics": (C.c_int, [_vp, _u32, _vp, _vp, _P(_d)]),
    "score_batch_rediscr_kinetics": (C.c_int, [_vp, _u32, _vp, _vp, _P(_d)]),
    "score_batch_rediscr_texture": (C.c_int, [_vp, _u32, _vp, _u32, _vp, _vp]),
    "score_batch_final_grain_sizes": (C.c_int, [_vp, _vp]),
    "score_percolation_analyze": (C.c_int, [_vp, C.c_int, _P(Percolation), _vp, _u32, _vp]),
    "score_batch_percolation_analyze": (C.c_int, [_vp, _u32, C.c_int, _P(Percolation), _vp, _u32, _vp]),
    "score_mobility_weight": (C.c_int, [_P(Params), _vp, _vp, _P(_d)]),
    "score_mobility_table_noalloc": (C.c_int, [_P(Params), _vp, _u32, _vp, _u32, _vp, _vp, _vp]),
    "score_gen_default": (C.c_int, [_P(GenParams)]),
    "score_generate_domain": (C.c_int, [_P(GenParams), _vp, _vp, _vp, _vp, _vp, _vp]),
    "score_generate_domain_gpu": (C.c_int, [_P(GenParams), _vp, _vp, _vp, _vp, _vp, _vp, C.c_int]),
}

_lib = None


def load(path: str | Path | None = None) -> C.CDLL:
    """Load libscore_gb300.so from the source tree (never a site-packages copy)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    if path is None:
        from .build import library_path
        path = library_path()
    path = Path(path)
    if not path.exists():
        raise RuntimeError(f"{path} is missing: run score_gb300.build.build() (or __graft_entry__.build()) first")
    lib = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


# entry points of the host-only library (host_api.cpp, host_generate.cpp)
HOST_FUNCTIONS = ("score_params_default", "score_uds_read", "score_mobility_weight", "score_gen_default", "score_generate_domain")
_host = None


def load_host() -> C.CDLL:
    """Load libscore_host.so (parameters, host mobility weight, domain generator; no CUDA)."""
    global _host
    if _host is not None:
        return _host
    from .build import host_library_path
    path = host_library_path()
    if not path.exists():
        raise RuntimeError(f"{path} is missing: run score_gb300.build.build() (or __graft_entry__.build()) first")
    lib = C.CDLL(str(path))
    for name in HOST_FUNCTIONS:
        fn = getattr(lib, name)
        fn.restype, fn.argtypes = SIGNATURES[name]
    _host = lib
    return lib


class ScoreError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"score_gb300 status {status}: {msg}")
        self.status = status
