"""Percolation analysis on the GPU (score_percolation_analyze): on growth fixtures stopped at
X = 0.01 ... 0.99, the reference mode equals the reference's own analysis (cluster count, largest,
spanning, sorted sizes) and, cell by cell, the oracle's restatement of the reference's scan; the
connected mode equals the oracle's true 6-connected clusters.  Also at 128^3 mid-run."""
import numpy as np
import pytest

import oracle
import score_gb300 as sg
from _golden import load_case, load_percolation

pytestmark = pytest.mark.gpu


def check(gm, d, bin_ref=None, ref_hdr=None, ref_sizes=None, tag=""):
    b = bin_ref if bin_ref is not None else None
    r = gm.percolation(labels=True)
    t = gm.percolation(connected=True, labels=True)
    if b is None:
        return r, t
    o_r = oracle.percolation(b, d.nx, d.ny, d.nz, reference_scan=True)
    o_t = oracle.percolation(b, d.nx, d.ny, d.nz)
    assert np.array_equal(r["labels"].ravel(), o_r["labels"]), f"reference-mode labels {tag}"
    assert np.array_equal(t["labels"].ravel(), o_t["labels"]), f"connected-mode labels {tag}"
    for got, want in ((r, o_r), (t, o_t)):
        assert (got["n_clusters"], got["largest"], got["percolates"], got["spans"]) == \
               (want["n_clusters"], want["largest"], want["percolates"], want["spans"]), tag
        assert np.array_equal(got["sizes"], want["sizes"]), tag
    if ref_hdr is not None:
        n, big, perc, _ = (int(v) for v in ref_hdr)
        assert (r["n_clusters"], r["largest"], int(r["percolates"])) == (n, big, perc), f"reference analysis {tag}"
        assert np.array_equal(r["sizes"], ref_sizes), f"reference size distribution {tag}"
        assert r["PL"] == big / d.ncells
    return r, t


def test_gpu_percolation_matches_reference(gpu, tmp_path):
    for c in load_percolation():
        _, d, _ = load_case(c["name"], tmp_path)
        uds = tmp_path / "p.uds"
        uds.write_text(c["uds"])
        p = sg.read_uds(uds)
        with sg.GrowthMachine(p, device=0) as gm:
            gm.load_domain(d)
            gm.place_nuclei()
            gm.run_until()
            check(gm, d, c["bin"][: d.ncells], c["hdr"], c["sizes"], f"{c['name']} X={c['x']}")


def test_gpu_percolation_at_128_mid_run(gpu, tmp_path):
    d = sg.generate_domain(128, 128, 128, 500, 200, seed=0)
    p = sg.read_uds(sg.UdsSpec(nx=128, ny=128, nz=128, xmax="0.3").write(tmp_path / "c0.uds"))
    sim = oracle.Sim(p, d)
    sim.advance()
    b = sim.binarize()
    sim.close()
    with sg.GrowthMachine(p, device=0) as gm:
        gm.load_domain(d)
        gm.place_nuclei()
        gm.run_until()
        r, t = check(gm, d, b, tag="128^3 X=0.3")
    assert r["n_clusters"] > 20 and r["n_clusters"] >= t["n_clusters"]


def test_gpu_percolation_odd_extents_mid_run(gpu, tmp_path):
    """Odd extents (padding words in the device grid's bricks) mid-run, against the oracle."""
    d = sg.generate_domain(45, 51, 37, 60, 40, seed=5)
    p = sg.read_uds(sg.UdsSpec(nx=45, ny=51, nz=37, xmax="0.4").write(tmp_path / "odd.uds"))
    sim = oracle.Sim(p, d)
    sim.advance()
    b = sim.binarize()
    sim.close()
    with sg.GrowthMachine(p, device=0) as gm:
        gm.load_domain(d)
        gm.place_nuclei()
        gm.run_until()
        check(gm, d, b, tag="45x51x37 X=0.4")
