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


def config_cases() -> list[str]:
    """Fixtures of the benchmark configurations (config0_128, config1_512)."""
    return sorted(p.stem for p in GOLDEN.glob("config*_*.npz"))


def input_digest(d) -> str:
    """SHA-256 over a domain's inputs, as tests/golden/make_golden.py computes it."""
    import hashlib
    h = hashlib.sha256()
    for a in (d.grid, d.defg_quat, d.defg_rho0, d.rxg_quat, d.rxg_site, d.rxg_tincub):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def labels_digest(labels) -> str:
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(labels, dtype=np.uint32).tobytes()).hexdigest()


def load_config(name: str, tmp_path: Path):
    """(params, domain, golden dict) of a benchmark-configuration fixture: the domain is
    regenerated from the stored generator arguments and checked against the stored
    input digest before anything is compared."""
    z = np.load(GOLDEN / f"{name}.npz")
    uds = tmp_path / f"{name}.uds"
    uds.write_text(str(z["uds"]))
    p = sg.read_uds(uds)
    n, ng, nn, seed = (int(v) for v in z["gen"])
    d = sg.generate_domain(n, n, n, ng, nn, seed=seed)
    assert input_digest(d) == str(z["input_sha256"]), "the generator no longer reproduces the fixture's inputs"
    g = {k: z[k] for k in TRACE_FIELDS}
    g["labels_sha256"] = str(z["labels_sha256"])
    g["rxg_counts"] = z["rxg_counts"]
    g["defg_counts"] = z["defg_counts"]
    return p, d, g


def load_evolution(tmp_path: Path):
    """The evolution-ensemble fixture: per domain (params, domain, reference log dict), plus the
    ensemble's rediscretization (tmax, nslots, nclass, kinetics, texture) made from the reference."""
    z = np.load(GOLDEN / "evolution_ensemble.npz")
    doms = []
    k = 0
    while f"d{k}_uds" in z:
        uds = tmp_path / f"evo{k}.uds"
        uds.write_text(str(z[f"d{k}_uds"]))
        p = sg.read_uds(uds)
        nx, ny, nz = (int(v) for v in z[f"d{k}_dims"])
        d = sg.Domain(nx, ny, nz, z[f"d{k}_grid"].astype(np.uint32).reshape(nz, ny, nx), z[f"d{k}_defg_quat"],
                      z[f"d{k}_defg_rho0"], z[f"d{k}_rxg_quat"], z[f"d{k}_rxg_site"], z[f"d{k}_rxg_tincub"])
        g = {a: z[f"d{k}_{a}"] for a in ("t_end", "cls", "snap_t", "snap_X", "snap_step", "snap_Sv", "snap_counts", "areas",
                                          "interp", "final")}
        g["t_end"] = float(g["t_end"])
        doms.append((p, d, g))
        k += 1
    ens = {a: z[a] for a in ("kinetics", "texture")}
    ens.update({"tmax": float(z["tmax"]), "nslots": int(z["nslots"]), "nclass": int(z["nclass"])})
    return doms, ens


def evo_descriptor(d, g) -> dict:
    """An oracle post-processing descriptor of a domain's reference log."""
    return {"ndefg": d.ndefg, "nrxg": d.nrxg, "t": g["snap_t"], "counts": g["snap_counts"], "final": g["final"],
            "tsimend": g["t_end"], "cells": d.ncells, "cls": g["cls"]}


def load_percolation():
    """The reference's percolation analyses: per (domain, X) the .uds, the binarized structure,
    (n clusters, largest, percolates, checkLabeling failed) and the ascending cluster sizes."""
    z = np.load(GOLDEN / "percolation.npz")
    out = []
    for c in z["cases"]:
        for k in range(len(z["xs"])):
            key = f"{c}_{k}"
            out.append({"name": str(c), "x": str(z["xs"][k]), "uds": str(z[f"{key}_uds"]), "hdr": z[f"{key}_hdr"],
                        "sizes": z[f"{key}_sizes"], "bin": np.unpackbits(z[f"{key}_bin"])})
    return out
