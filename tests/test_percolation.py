"""Percolation analysis, CPU side (SCORE_PercAnalyzer.cpp, log_PERCOLATION): the oracle against the
reference's own analysis of growth fixtures stopped at X = 0.01 ... 0.99 (binarized structure, cluster
count, largest cluster, spanning, sorted cluster sizes), bit for bit; and the reference's scan against
the true 6-connected clusters."""
import numpy as np

import oracle
import score_gb300 as sg
from _golden import load_case, load_percolation


def test_oracle_binarization_and_reference_scan_match_reference(built, tmp_path):
    cases = load_percolation()
    assert len(cases) == 24
    splits = 0
    for c in cases:
        p0, d, _ = load_case(c["name"], tmp_path)
        uds = tmp_path / "p.uds"
        uds.write_text(c["uds"])
        p = sg.read_uds(uds)
        sim = oracle.Sim(p, d)
        sim.advance()
        b = sim.binarize()
        sim.close()
        assert np.array_equal(b, c["bin"][: b.size]), (c["name"], c["x"])
        r = oracle.percolation(b, d.nx, d.ny, d.nz, reference_scan=True)
        n, big, perc, split = (int(v) for v in c["hdr"])
        assert (r["n_clusters"], r["largest"], int(r["percolates"])) == (n, big, perc), (c["name"], c["x"])
        assert np.array_equal(r["sizes"], c["sizes"]), (c["name"], c["x"])
        # the reference's labeling check fails exactly where its scan split a true cluster
        t = oracle.percolation(b, d.nx, d.ny, d.nz, reference_scan=False)
        assert (t["n_clusters"] < n) == bool(split), (c["name"], c["x"], t["n_clusters"], n, split)
        splits += split
    assert splits > 0  # the fixtures exercise the reference's split clusters


def test_true_clusters_are_6_connected_components(built):
    """The true-cluster mode against a breadth-first search on random structures, with the origin
    cell left out of every cluster as in the reference."""
    rng = np.random.default_rng(3)
    for shape, p in [((17, 13, 11), 0.3), ((20, 20, 20), 0.55), ((9, 31, 7), 0.7)]:
        nx, ny, nz = shape
        b = (rng.random(nx * ny * nz) < p).astype(np.uint8)
        b[0] = 1
        r = oracle.percolation(b, nx, ny, nz)
        lab = np.zeros(nx * ny * nz, dtype=np.int64)
        seen = np.zeros_like(b, dtype=bool)
        seen[0] = True
        nxt = 0
        for s in range(nx * ny * nz):
            if not b[s] or seen[s]:
                continue
            nxt += 1
            stack = [s]
            seen[s] = True
            while stack:
                c = stack.pop()
                lab[c] = nxt
                x, y, z = c % nx, (c // nx) % ny, c // (nx * ny)
                for dx, dy, dz in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
                    X, Y, Z = x + dx, y + dy, z + dz
                    if 0 <= X < nx and 0 <= Y < ny and 0 <= Z < nz:
                        q = X + nx * (Y + ny * Z)
                        if b[q] and not seen[q]:
                            seen[q] = True
                            stack.append(q)
        assert np.array_equal(r["labels"], lab) and r["n_clusters"] == nxt
