"""Generate the golden fixtures of tests/golden/ from the SCORE reference itself.

Each growth case: a small synthetic domain (this package's deterministic generator; the reference
accepts edges of 50 cells and more, SCORE_Defs_Functionality.h:84),
a .uds parameter file (UdsSpec), and the reference's own growth loop run on them by
the harness in oracle/ref (reference sources compiled by oracle/ref/Makefile,
OMP_NUM_THREADS=1, the canonical order).  The fixture stores the inputs (the .uds
text and the domain arrays, so tests do not depend on the generator) and the
reference's per-step trace and final labels.

The ptab case stores the reference's mobility weights P(rxg, defg) for every pair
(reg_calc_mobilityweight, SCORE_Kernel.cpp:2460-2527) of a small grain set.

The two benchmark-configuration cases run the reference on the full-size domains of the
benchmark: config 0 (128^3, 500 Voronoi grains, 200 site-saturated nuclei) and config 1
(512^3, 20,000 grains, 50,000 nuclei: the headline workload's domain, seed 0).  Their
inputs are too large to store, so the fixture keeps the generator arguments and a
SHA-256 of the generated inputs (the generator gives identical bits on x86-64 and
aarch64), the reference's full per-step trace, a SHA-256 of its final labels and its
per-grain cell counts.

Run from the repository root, with the reference sources at $SCORE_REFERENCE:
    python tests/golden/make_golden.py            # every case
    python tests/golden/make_golden.py config0    # only the named cases
"""
from __future__ import annotations

import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
import score_gb300 as sg  # noqa: E402

# name: (UdsSpec overrides, (nx, ny, nz, grains, nuclei, seed), generator overrides)
CASES = {
    "base": ({}, (50, 50, 50, 20, 12, 101), {}),
    "noncubic": ({}, (50, 64, 56, 30, 20, 102), {}),
    "distinct_mob": ({"LAGBm0": "30.0", "GSm0": "600.0"}, (50, 50, 50, 30, 24, 103), {}),
    "rollett_holm": ({"mobility_model": 2}, (50, 50, 50, 30, 24, 104), {}),
    "defrag": ({"defragmentation": 1, "defrag_x": ["0.2", "0.5", "0.8"]}, (50, 50, 50, 25, 16, 105), {}),
    "recovery_mp": ({"recovery": 3}, (50, 50, 50, 25, 16, 106), {}),
    "zener_timedep": ({"zener": 2, "zener_table": [("0.0", "0.0"), ("0.1", "4.0e5"), ("360000.0", "4.0e5")]},
                      (50, 50, 50, 25, 16, 107), {}),
    "heating": ({"schedule": [("0.0", "700.0"), ("0.05", "760.0"), ("360000.0", "760.0")]}, (50, 50, 50, 25, 16, 108), {}),
    "many_nuclei_small_cache": ({"initial_cache": "0.05"}, (56, 56, 56, 30, 150, 109), {}),
    "texture_bimodal": ({}, (50, 50, 50, 40, 30, 110),
                        {"ori_mode": 1, "ncomp": 3, "scatter_deg": 10.0, "rho_mode": 1, "rho_lo": 1e14, "rho_hi": 5e15}),
}
PTAB = (40, 80, 111)  # nrxg, ndefg, seed
# ensemble of the on-the-fly characterization and post-processing fixture: per domain (nx, ny, nz, grains,
# nuclei, seed); logpoints, RX area threshold, rediscretization slots, orientation classes
EVO_DOMAINS = [(50, 50, 50, 20, 12, 201), (56, 50, 52, 30, 24, 202), (50, 54, 50, 25, 40, 203)]
EVO_LOGPOINTS = ["0.0", "0.05", "0.1", "0.2", "0.35", "0.5", "0.65", "0.8", "0.9", "0.95"]
EVO_AREA, EVO_SLOTS, EVO_CLASSES = 13, 40, 4
# percolation fixture: cubic growth fixtures stopped at these X, analysed by the reference
PERC_CASES = ["base", "many_nuclei_small_cache", "texture_bimodal", "rollett_holm"]
PERC_X = ["0.01", "0.05", "0.15", "0.3", "0.6", "0.99"]
# benchmark configurations: name -> (edge, grains, nuclei, seed)
CONFIGS = {"config0": (128, 500, 200, 0), "config1": (512, 20000, 50000, 0)}


def narrow(a: np.ndarray) -> np.ndarray:
    """u32 ids stored as u16 when they fit (the tests widen them again)."""
    return a.astype(np.uint16) if a.size and int(a.max()) < 65536 else a


def domain_arrays(d: sg.Domain) -> dict:
    return {"dims": np.array([d.nx, d.ny, d.nz], dtype=np.uint32), "grid": narrow(d.grid), "defg_quat": d.defg_quat,
            "defg_rho0": d.defg_rho0, "rxg_quat": d.rxg_quat, "rxg_site": d.rxg_site, "rxg_tincub": d.rxg_tincub}


def make_case(name: str, kw: dict, geo: tuple, gkw: dict, wd: Path) -> Path:
    nx, ny, nz, ng, nn, seed = geo
    d = sg.generate_domain(nx, ny, nz, ng, nn, seed=seed, **gkw)
    spec = sg.UdsSpec(nx=nx, ny=ny, nz=nz, **kw)
    uds = spec.write(wd / f"{name}.uds")
    r = oracle.run_ref("loop", uds, d, workdir=wd / name)
    tr = r["trace"][1:]  # record 0 is the state before the first step
    out = HERE / f"growth_{name}.npz"
    np.savez_compressed(
        out, uds=np.array(spec.text()), **domain_arrays(d),
        t=tr["t"], dt=tr["dt"], Xcells=tr["Xcells"], Sv=tr["Sv"], n_full=tr["nfull"], Pmax=tr["Pmax"], rhomax=tr["rhomax"],
        labels=narrow(r["labels"]),
        rxg_counts=np.array([r["rxg"].get(i, 0) for i in range(d.nrxg)], dtype=np.uint32),
        defg_counts=np.array([r["defg"].get(i, 0) for i in range(d.ndefg)], dtype=np.uint32))
    print(f"{out.name}: {len(tr)} steps, X={tr['Xcells'][-1] / d.ncells:.4f}, {out.stat().st_size // 1024} KiB")
    return out


def input_digest(d: sg.Domain) -> str:
    """SHA-256 over the generated inputs (grid, orientations, rho, nucleus sites and times)."""
    import hashlib
    h = hashlib.sha256()
    for a in (d.grid, d.defg_quat, d.defg_rho0, d.rxg_quat, d.rxg_site, d.rxg_tincub):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def make_config(name: str, wd: Path) -> Path:
    import hashlib
    n, ng, nn, seed = CONFIGS[name]
    d = sg.generate_domain(n, n, n, ng, nn, seed=seed)
    spec = sg.UdsSpec(nx=n, ny=n, nz=n)
    uds = spec.write(wd / f"{name}.uds")
    r = oracle.run_ref("loop", uds, d, workdir=wd / name)
    tr = r["trace"][1:]
    out = HERE / f"{name}_{n}.npz"
    np.savez_compressed(
        out, uds=np.array(spec.text()), gen=np.array([n, ng, nn, seed], dtype=np.int64), input_sha256=np.array(input_digest(d)),
        t=tr["t"], dt=tr["dt"], Xcells=tr["Xcells"], Sv=tr["Sv"], n_full=tr["nfull"], Pmax=tr["Pmax"], rhomax=tr["rhomax"],
        labels_sha256=np.array(hashlib.sha256(np.ascontiguousarray(r["labels"], dtype=np.uint32).tobytes()).hexdigest()),
        rxg_counts=np.array([r["rxg"].get(i, 0) for i in range(d.nrxg)], dtype=np.uint32),
        defg_counts=np.array([r["defg"].get(i, 0) for i in range(d.ndefg)], dtype=np.uint32))
    print(f"{out.name}: {len(tr)} steps, X={tr['Xcells'][-1] / d.ncells:.4f}, {out.stat().st_size // 1024} KiB")
    return out


def read_evo(wd: Path, d: sg.Domain):
    """Snapshots (t, X, step, Sv, counts) and RX area profiles the harness wrote."""
    G = d.ndefg + d.nrxg
    raw = (wd / "out.grainevo").read_bytes()
    rec = 24 + 4 * G
    snaps = []
    for i in range(len(raw) // rec):
        t, X = np.frombuffer(raw[i * rec:i * rec + 16], dtype=np.float64)
        st, sv = np.frombuffer(raw[i * rec + 16:i * rec + 24], dtype=np.uint32)
        snaps.append((t, X, st, sv, np.frombuffer(raw[i * rec + 24:(i + 1) * rec], dtype=np.uint32)))
    raw = (wd / "out.rxprofile").read_bytes()
    rec = 24 + 8 * d.nz
    areas = [np.frombuffer(raw[i * rec + 24:(i + 1) * rec], dtype=np.uint32).reshape(d.nz, 2) for i in range(len(raw) // rec)]
    return snaps, areas


def make_evo(wd: Path) -> Path:
    """Grain-evolution log, RX area profiles and ensemble post-processing of a 3-domain ensemble, all
    from the reference: its log_grainevo / log_rxareaprofile at the logpoints and its
    get_interpCellCount at the rediscretized times; the ensemble sums are formed from those values in
    the order of postprocess_rediscr_kinetics / postprocess_rediscr_macrotexture."""
    import os
    doms, specs = [], []
    for k, (nx, ny, nz, ng, nn, seed) in enumerate(EVO_DOMAINS):
        doms.append(sg.generate_domain(nx, ny, nz, ng, nn, seed=seed))
        specs.append(sg.UdsSpec(nx=nx, ny=ny, nz=nz, logpoints=EVO_LOGPOINTS, area_threshold=EVO_AREA))
    os.environ["SCORE_LOG_AREA"] = str(EVO_AREA)
    first = [oracle.run_ref("loop", specs[k].write(wd / f"evo{k}.uds"), d, workdir=wd / f"evo{k}")
             for k, d in enumerate(doms)]
    tmax = 0.0
    for r in first:
        t_end = float.fromhex(r["t_end"])
        if t_end >= tmax:
            tmax = t_end
    os.environ["SCORE_REDISCR"] = f"{EVO_SLOTS} {tmax!r}"
    out = {"tmax": np.array(tmax), "nslots": np.array(EVO_SLOTS), "nclass": np.array(EVO_CLASSES),
           "area_threshold": np.array(EVO_AREA)}
    rng = np.random.default_rng(7)
    kin = np.zeros(EVO_SLOTS)
    tex = np.zeros((EVO_SLOTS, EVO_CLASSES))
    for k, d in enumerate(doms):
        r = oracle.run_ref("loop", wd / f"evo{k}.uds", d, workdir=wd / f"evo{k}b")
        snaps, areas = read_evo(r["workdir"], d)
        G = d.ndefg + d.nrxg
        interp = np.fromfile(r["workdir"] / "out.interp", dtype=np.float64).reshape(EVO_SLOTS, G)
        cls = rng.integers(0, EVO_CLASSES, size=G).astype(np.uint32)
        # postprocess_rediscr_kinetics (SCORE_SolitaryUnitAveraging.cpp:576-600): sums in grain order
        for n in range(EVO_SLOTS):
            dv = 0.0
            for g in range(d.ndefg):
                dv = dv + float(interp[n, g])
            kin[n] = kin[n] + (float(d.ncells) - dv)
        # postprocess_rediscr_macrotexture (:705-747): deformed then rx grains, per class
        for n in range(EVO_SLOTS):
            acc = [0.0] * EVO_CLASSES
            for g in range(G):
                acc[cls[g]] += float(interp[n, g])
            for c in range(EVO_CLASSES):
                tex[n, c] += acc[c]
        out.update({f"d{k}_uds": np.array(specs[k].text()), **{f"d{k}_{a}": b for a, b in domain_arrays(d).items()},
                    f"d{k}_t_end": np.array(float.fromhex(r["t_end"])), f"d{k}_cls": cls,
                    f"d{k}_snap_t": np.array([x[0] for x in snaps]), f"d{k}_snap_X": np.array([x[1] for x in snaps]),
                    f"d{k}_snap_step": np.array([x[2] for x in snaps], dtype=np.uint32),
                    f"d{k}_snap_Sv": np.array([x[3] for x in snaps], dtype=np.uint32),
                    f"d{k}_snap_counts": np.array([x[4] for x in snaps]), f"d{k}_areas": np.array(areas),
                    f"d{k}_interp": interp,
                    f"d{k}_final": np.array([r["defg"].get(i, 0) for i in range(d.ndefg)] + [r["rxg"].get(i, 0) for i in range(d.nrxg)],
                                            dtype=np.uint32)})
    del os.environ["SCORE_LOG_AREA"], os.environ["SCORE_REDISCR"]
    out["kinetics"] = kin
    out["texture"] = tex
    path = HERE / "evolution_ensemble.npz"
    np.savez_compressed(path, **out)
    print(f"{path.name}: {len(doms)} domains, {[len(read_evo(wd / f'evo{k}b', doms[k])[0]) for k in range(len(doms))]} snapshots, "
          f"{path.stat().st_size // 1024} KiB")
    return path


def make_perc(wd: Path) -> Path:
    """The reference's percolation analysis (log_PERCOLATION: binarize, Hoshen-Kopelman, compactify,
    checkLabeling, percolates, cluster-size distribution) of growth fixtures stopped at several X."""
    import os
    out = {}
    os.environ["SCORE_PERC"] = "1"
    for name in PERC_CASES:
        z = np.load(HERE / f"growth_{name}.npz")
        nx, ny, nz = (int(v) for v in z["dims"])
        d = sg.Domain(nx, ny, nz, z["grid"].astype(np.uint32).reshape(nz, ny, nx), z["defg_quat"], z["defg_rho0"],
                      z["rxg_quat"], z["rxg_site"], z["rxg_tincub"])
        base = str(z["uds"])
        for k, xm in enumerate(PERC_X):
            uds = wd / f"perc_{name}_{k}.uds"
            uds.write_text(base.replace('"XMAX"\t"0.99"', f'"XMAX"\t"{xm}"'))
            r = oracle.run_ref("loop", uds, d, workdir=wd / f"perc_{name}_{k}")
            raw = (r["workdir"] / "out.perc").read_bytes()
            n, big, perc, split = (int(v) for v in np.frombuffer(raw[:16], dtype=np.uint32))
            key = f"{name}_{k}"
            out[f"{key}_uds"] = np.array(uds.read_text())
            out[f"{key}_hdr"] = np.array([n, big, perc, split], dtype=np.uint32)
            out[f"{key}_sizes"] = np.frombuffer(raw[16:16 + 4 * n], dtype=np.uint32)
            out[f"{key}_bin"] = np.packbits(np.frombuffer(raw[16 + 4 * n:], dtype=np.uint8))
    del os.environ["SCORE_PERC"]
    out["cases"] = np.array(PERC_CASES)
    out["xs"] = np.array(PERC_X)
    path = HERE / "percolation.npz"
    np.savez_compressed(path, **out)
    print(f"{path.name}: {len(PERC_CASES)} domains x {len(PERC_X)} X, {path.stat().st_size // 1024} KiB")
    return path


def make_ptab(wd: Path) -> Path:
    nrxg, ndefg, seed = PTAB
    d = sg.generate_domain(50, 50, 50, ndefg, nrxg, seed=seed)
    out = {}
    for model in (1, 2):
        spec = sg.UdsSpec(nx=50, ny=50, nz=50, mobility_model=model)
        uds = spec.write(wd / f"ptab{model}.uds")
        r = oracle.run_ref("ptab", uds, d, workdir=wd / f"ptab{model}")
        out[f"uds{model}"] = np.array(spec.text())
        out[f"P{model}"] = r["ptab"]
    path = HERE / "mobility_weights.npz"
    np.savez_compressed(path, defg_quat=d.defg_quat, rxg_quat=d.rxg_quat, **out)
    print(f"{path.name}: {nrxg}x{ndefg} pairs, {path.stat().st_size // 1024} KiB")
    return path


def main() -> None:
    if not oracle.reference_available():
        sys.exit("the reference sources are required to generate the golden fixtures")
    oracle.build_ref()
    only = set(sys.argv[1:])
    with tempfile.TemporaryDirectory() as td:
        wd = Path(td)
        for name, (kw, geo, gkw) in CASES.items():
            if not only or name in only:
                make_case(name, kw, geo, gkw, wd)
        if not only or "ptab" in only:
            make_ptab(wd)
        if not only or "evo" in only:
            make_evo(wd)
        if not only or "perc" in only:
            make_perc(wd)
        for name in CONFIGS:
            if not only or name in only:
                make_config(name, wd)


if __name__ == "__main__":
    main()
