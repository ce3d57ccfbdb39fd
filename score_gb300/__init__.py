"""score_gb300 — GB300-native recrystallization growth step of SCORE.

The growth step (front-cell fill update, 26-neighbour infection with overshoot
carry, slot recycling, adaptive dt) runs as hand-written sm_103a CUDA kernels
behind the C ABI in include/score_gb300.h; this package is the Python mirror of
that boundary: one domain (GrowthMachine) or a batched ensemble of independent
domains (Batch).
"""
from .build import build, library_path
from ._abi import Params, StepStats, Timing, Tune, GenParams, ScoreError
from .growth import (Batch, Domain, GrowthMachine, UdsSpec, default_params, generate_domain, mobility_weight, read_uds,
                     stats_dict)

__all__ = ["build", "library_path", "Params", "StepStats", "Timing", "Tune", "GenParams", "ScoreError", "Batch", "Domain",
           "GrowthMachine", "UdsSpec", "default_params", "generate_domain", "mobility_weight", "read_uds", "stats_dict"]
