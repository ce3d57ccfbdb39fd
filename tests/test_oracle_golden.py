"""The CPU oracle pinned against the reference: every golden fixture (the
reference's own growth loop on small domains, tests/golden/) must be reproduced
bit for bit — per-step t, dt, X cells, Sv, full cells, P max and rho max, the final
labels and the per-grain cell counts — and the host mobility weight must equal the
reference's P(rxg, defg) for every stored pair."""
import numpy as np
import pytest

import oracle
import score_gb300 as sg
from _golden import (GOLDEN, TRACE_FIELDS, config_cases, first_difference, growth_cases, labels_digest, load_case,
                     load_config)


@pytest.mark.parametrize("name", growth_cases())
def test_oracle_reproduces_reference(built, tmp_path, name):
    p, d, g = load_case(name, tmp_path)
    r = oracle.run(p, d)
    tr = r["trace"]
    assert r["status"] == 0
    for f in TRACE_FIELDS:
        assert np.array_equal(tr[f], g[f]), f"{f}: {first_difference(tr[f], g[f])}"
    assert np.array_equal(r["labels"], g["labels"]), "final labels"
    assert np.array_equal(r["rxg_counts"], g["rxg_counts"]) and np.array_equal(r["defg_counts"], g["defg_counts"])


def test_golden_set_is_complete():
    assert len(growth_cases()) >= 10
    assert (GOLDEN / "mobility_weights.npz").exists()
    assert config_cases() == ["config0_128", "config1_512"]


@pytest.mark.parametrize("name", ["config0_128", pytest.param("config1_512", marks=pytest.mark.slow)])
def test_oracle_reproduces_reference_at_benchmark_size(built, tmp_path, name):
    """The benchmark configurations themselves (128^3 / 500 grains / 200 nuclei, and the
    512^3 / 20,000 grains / 50,000 nuclei headline domain), run by the reference's growth
    loop: per-step trace, final labels (SHA-256) and per-grain counts, bit for bit."""
    p, d, g = load_config(name, tmp_path)
    r = oracle.run(p, d)
    assert r["status"] == 0
    tr = r["trace"]
    for f in TRACE_FIELDS:
        assert np.array_equal(tr[f], g[f]), f"{f}: {first_difference(tr[f], g[f])}"
    assert labels_digest(r["labels"]) == g["labels_sha256"], "final labels"
    assert np.array_equal(r["rxg_counts"], g["rxg_counts"]) and np.array_equal(r["defg_counts"], g["defg_counts"])


@pytest.mark.skipif(not oracle.reference_available(), reason="reference sources not found (SCORE_REFERENCE unset, no prebuilt harness)")
@pytest.mark.parametrize("name", ["base", "rollett_holm"])
def test_harness_replay_matches_unmodified_solve(built, tmp_path, name):
    """The fixtures come from the harness's replay of solve_RXGROWTH (without its logging);
    the unmodified caHdl::solve_RXGROWTH (SCORE_Kernel.cpp:6497-6792) must end at the same
    time (bit for bit), after the same number of steps, with the same per-grain counts."""
    p, d, g = load_case(name, tmp_path)
    uds = tmp_path / f"{name}.uds"
    asis = oracle.run_ref("asis", uds, d, workdir=tmp_path / "asis")
    loop = oracle.run_ref("loop", uds, d, workdir=tmp_path / "loop")
    assert asis["t_end"] == loop["t_end"], (asis["t_end"], loop["t_end"])
    assert int(asis["step_end"]) == int(loop["steps"]) == len(g["t"])
    assert float.fromhex(asis["t_end"]) == g["t"][-1]
    assert asis["rxg"] == loop["rxg"] and asis["defg"] == loop["defg"]
    assert [asis["rxg"][i] for i in range(d.nrxg)] == list(g["rxg_counts"])


@pytest.mark.parametrize("model", [1, 2])
def test_mobility_weight_matches_reference(built, tmp_path, model):
    z = np.load(GOLDEN / "mobility_weights.npz")
    uds = tmp_path / "p.uds"
    uds.write_text(str(z[f"uds{model}"]))
    p = sg.read_uds(uds)
    ref = z[f"P{model}"]
    qr, qd = z["rxg_quat"], z["defg_quat"]
    host = np.array([[sg.mobility_weight(p, qr[i], qd[j]) for j in range(len(qd))] for i in range(len(qr))])
    orc = np.array([[oracle.mobility_weight(p, qr[i], qd[j]) for j in range(len(qd))] for i in range(len(qr))])
    assert np.array_equal(host, ref)
    assert np.array_equal(orc, ref)
    if model == 1:
        assert (ref == -1.0).any() or (ref == 0.0).any()


@pytest.mark.skipif(not oracle.reference_available(), reason="reference sources not present on this machine")
@pytest.mark.parametrize("uds_kw,gen_kw", [
    ({}, {}),
    ({"mobility_model": 2, "initial_cache": "0.04"}, {"ori_mode": 1, "ncomp": 2, "scatter_deg": 15.0}),
])
def test_oracle_matches_live_reference(built, tmp_path, uds_kw, gen_kw):
    """A case outside the fixtures, run through the compiled reference here."""
    d = sg.generate_domain(52, 50, 54, 35, 40, seed=4242, **gen_kw)
    uds = sg.UdsSpec(nx=52, ny=50, nz=54, **uds_kw).write(tmp_path / "live.uds")
    p = sg.read_uds(uds)
    ref = oracle.run_ref("loop", uds, d, workdir=tmp_path / "ref")
    rt = ref["trace"][1:]
    tr = oracle.run(p, d)["trace"]
    for f, rf in [("t", "t"), ("dt", "dt"), ("Xcells", "Xcells"), ("Sv", "Sv"), ("n_full", "nfull"), ("Pmax", "Pmax"),
                  ("rhomax", "rhomax")]:
        assert np.array_equal(tr[f], rt[rf]), f"{f}: {first_difference(tr[f], rt[rf])}"
    assert np.array_equal(oracle.run(p, d)["labels"], ref["labels"])


def test_host_weight_matches_oracle_on_random_and_boundary_pairs(built, tmp_path):
    """The library's host weight (which skips the 40deg<111> deviation far from 40 deg) against
    the oracle's restatement, bit for bit: random orientation pairs, and pairs rotated to lie
    just inside and outside the 15 deg and the 30 / 50 deg (40 +- 10) thresholds."""
    rng = np.random.default_rng(7)
    p = sg.read_uds(sg.UdsSpec(nx=50, ny=50, nz=50).write(tmp_path / "w.uds"))

    def unit(q):
        return q / np.linalg.norm(q, axis=-1, keepdims=True)

    def axis_angle(axis, deg):
        axis = unit(np.asarray(axis, dtype=np.float64))
        h = np.radians(deg) / 2.0
        return np.concatenate([np.cos(h)[..., None], np.sin(h)[..., None] * axis], axis=-1)

    def qmul(a, b):
        a0, a1, a2, a3 = np.moveaxis(a, -1, 0)
        b0, b1, b2, b3 = np.moveaxis(b, -1, 0)
        return np.stack([a0 * b0 - a1 * b1 - a2 * b2 - a3 * b3, a0 * b1 + a1 * b0 + a2 * b3 - a3 * b2,
                         a0 * b2 - a1 * b3 + a2 * b0 + a3 * b1, a0 * b3 + a1 * b2 - a2 * b1 + a3 * b0], axis=-1)

    qd = unit(rng.normal(size=(3000, 4)))
    qr = unit(rng.normal(size=(3000, 4)))
    # near the thresholds: rotations about random axes and about <111> by 15, 30, 40, 50 deg +- tiny
    k = 1200
    angles = rng.choice([15.0, 30.0, 50.0, 40.0], size=k) + rng.choice([-1e-7, 1e-7, -1e-4, 1e-4, 0.0], size=k)
    axes = np.where(rng.random((k, 1)) < 0.5, np.ones((k, 3)) + rng.normal(scale=1e-3, size=(k, 3)), rng.normal(size=(k, 3)))
    qr[:k] = unit(qmul(qd[:k], axis_angle(axes, angles)))
    host = np.array([sg.mobility_weight(p, qr[i], qd[i]) for i in range(len(qr))])
    orc = np.array([oracle.mobility_weight(p, qr[i], qd[i]) for i in range(len(qr))])
    assert np.array_equal(host.view(np.uint64), orc.view(np.uint64))
    assert (host == -1.0).any() and (host == 0.0).any() and ((host > 0.0) & (host < 1.0)).any()


def test_oracle_in_pieces_equals_one_run(built, tmp_path):
    """The bounded-sample form of the oracle (advance in pieces, as the CPU timing of the
    benchmark uses it) gives exactly the one-call run: trace, labels, counts."""
    p, d, g = load_case("base", tmp_path)
    whole = oracle.run(p, d)
    sim = oracle.Sim(p, d)
    parts = [sim.advance(x_target=0.99 * k / 7) for k in range(1, 8)] + [sim.advance(max_steps=5), sim.advance()]
    assert sim.done()
    tr = np.concatenate([q["trace"] for q in parts])
    assert all(q["status"] == 0 for q in parts)
    assert np.array_equal(tr, whole["trace"])
    fin = sim.finish()
    sim.close()
    assert np.array_equal(fin["labels"], whole["labels"]) and np.array_equal(fin["labels"], g["labels"])
    assert np.array_equal(fin["rxg_counts"], whole["rxg_counts"]) and np.array_equal(fin["defg_counts"], whole["defg_counts"])
