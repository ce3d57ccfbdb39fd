"""Loader of the golden fixtures in tests/golden/ (made by tests/golden/make_golden.py
from the SCORE reference's own growth loop)."""
from __future__ import annotations

from pathlib import Path

import numpy as np

import score_gb300 as sg

GOLDEN = Path(__file__).resolve().parent / "golden"
TRACE_FIELDS = ["t", "dt", "Xcells", "Sv", "n_full", "Pmax", "rhomax"]


def growth_cases() -> list[str]:
    return sorted(p.stem[len("growth_"):] for p in GOLDEN.glob("growth_*.npz"))


def load_case(name: str, tmp_path: Path):
    """(params, domain, golden dict) of fixture `name`."""
    z = np.load(GOLDEN / f"growth_{name}.npz")
    uds = tmp_path / f"{name}.uds"
    uds.write_text(str(z["uds"]))
    p = sg.read_uds(uds)
    nx, ny, nz = (int(v) for v in z["dims"])
    d = sg.Domain(nx, ny, nz, z["grid"].astype(np.uint32).reshape(nz, ny, nx), z["defg_quat"], z["defg_rho0"],
                  z["rxg_quat"], z["rxg_site"], z["rxg_tincub"])
    g = {k: z[k] for k in TRACE_FIELDS}
    g["labels"] = z["labels"].astype(np.uint32)
    g["rxg_counts"] = z["rxg_counts"]
    g["defg_counts"] = z["defg_counts"]
    return p, d, g


def first_difference(a: np.ndarray, b: np.ndarray) -> str:
    m = min(len(a), len(b))
    if len(a) != len(b) and np.array_equal(a[:m], b[:m]):
        return f"lengths {len(a)} vs {len(b)}"
    i = int(np.argmax(a[:m] != b[:m]))
    return f"step {i}: {a[i]!r} vs {b[i]!r}"
