"""Batched ensemble and launch configuration on the GPU.

A batch steps independent domains of different sizes and parameters in one sequence
of launches per step; every domain must still reproduce, bit for bit, what it gives
alone — the reference's own golden outputs, or the oracle.  The launch configuration
(tile size, grid sizes, graph or direct launches) must not change any result.
"""
import numpy as np
import pytest

import oracle
import score_gb300 as sg
from _golden import TRACE_FIELDS, first_difference, load_case

pytestmark = pytest.mark.gpu

TRACE_ATTR = {"t": "t", "dt": "dt", "Xcells": "Xcells", "Sv": "Sv", "n_full": "n_full", "Pmax": "Pmax", "rhomax": "rhomax"}


def assert_trace(tr, ref: dict, what: str):
    for f in TRACE_FIELDS:
        a = np.array([getattr(s, TRACE_ATTR[f]) for s in tr])
        assert np.array_equal(a, ref[f]), f"{what} {f}: {first_difference(a, ref[f])}"


def oracle_ref(p, d):
    r = oracle.run(p, d)
    t = r["trace"]
    return {f: t[f] for f in TRACE_FIELDS} | {"labels": r["labels"], "rxg_counts": r["rxg_counts"],
                                              "defg_counts": r["defg_counts"]}


def test_batch_of_golden_cases_matches_reference(gpu, tmp_path):
    names = ["base", "noncubic", "rollett_holm", "recovery_mp", "heating", "many_nuclei_small_cache", "defrag"]
    cases = [load_case(n, tmp_path) for n in names]
    with sg.Batch([p for p, _, _ in cases]) as b:
        for i, (_, d, _) in enumerate(cases):
            b.load_domain(i, d)
        b.place_nuclei()
        steps = b.run_until()
        assert steps == max(len(g["t"]) for _, _, g in cases)
        for i, (name, (_, d, g)) in enumerate(zip(names, cases)):
            assert_trace(b.trace(i), g, name)
            assert np.array_equal(b.labels(i).ravel(), g["labels"]), f"{name}: labels"
            rc, dc = b.grain_counts(i)
            assert np.array_equal(rc, g["rxg_counts"]) and np.array_equal(dc, g["defg_counts"]), name


def test_uneven_batch_matches_each_domain_alone(gpu, tmp_path):
    geo = [(64, 50, 72, 40, 30, 1), (50, 50, 50, 10, 5, 2), (90, 64, 52, 120, 80, 3), (56, 77, 61, 60, 200, 4),
           (50, 96, 50, 30, 20, 5)]
    params, doms = [], []
    for k, (nx, ny, nz, ng, nn, seed) in enumerate(geo):
        kw = {"mobility_model": 2} if k == 3 else ({"LAGBm0": "30.0", "GSm0": "600.0"} if k == 1 else {})
        params.append(sg.read_uds(sg.UdsSpec(nx=nx, ny=ny, nz=nz, **kw).write(tmp_path / f"d{k}.uds")))
        doms.append(sg.generate_domain(nx, ny, nz, ng, nn, seed=seed))
    with sg.Batch(params) as b:
        for i, d in enumerate(doms):
            b.load_domain(i, d)
        for rep in range(2):  # a restart replays the same bits
            if rep:
                b.restart()
            b.place_nuclei()
            b.run_until()
            for i, (p, d) in enumerate(zip(params, doms)):
                ref = oracle_ref(p, d)
                assert_trace(b.trace(i), ref, f"domain {i}")
                assert np.array_equal(b.labels(i).ravel(), ref["labels"]), f"domain {i}: labels"


def run_single(p, d, **tune):
    with sg.GrowthMachine(p) as gm:
        gm.load_domain(d)
        if tune:
            gm.set_tune(**tune)
        gm.place_nuclei()
        tr = gm.run_until()
        return tr, gm.labels()


@pytest.mark.parametrize("tune", [
    dict(items=4, fill_blocks_per_sm=4, claim_blocks_per_sm=2, commit_blocks_per_sm=16, use_graph=0, spec_holes_pct=0),
    dict(items=16, fill_blocks_per_sm=32, claim_blocks_per_sm=16, commit_blocks_per_sm=2, use_graph=1, spec_holes_pct=100),
    dict(items=8, fill_blocks_per_sm=1, claim_blocks_per_sm=1, commit_blocks_per_sm=1, use_graph=1, spec_holes_pct=100),
    # the gathered-slot fill on every step, at 8 and 16 items
    dict(items=8, fill_blocks_per_sm=16, claim_blocks_per_sm=2, commit_blocks_per_sm=8, use_graph=1, spec_holes_pct=0),
    dict(items=16, fill_blocks_per_sm=8, claim_blocks_per_sm=4, commit_blocks_per_sm=4, use_graph=0, spec_holes_pct=0),
])
def test_launch_configuration_does_not_change_results(gpu, tmp_path, tune):
    p, d, g = load_case("texture_bimodal", tmp_path)
    tr, lab = run_single(p, d, **tune)
    assert_trace(tr, g, str(tune))
    assert np.array_equal(lab.ravel(), g["labels"])


def test_autotune_then_run(gpu, tmp_path):
    p, d, g = load_case("distinct_mob", tmp_path)
    with sg.GrowthMachine(p) as gm:
        gm.load_domain(d)
        t = gm.autotune()
        assert t.items in (4, 8, 16) and t.steps == len(g["t"])
        assert t.fill_ns_per_slot > 0 and t.claim_ns_per_cell > 0 and t.commit_ns_per_cell > 0
        tr = gm.run_until()  # autotune left it restarted with its nuclei placed
        assert_trace(tr, g, "after autotune")
        assert np.array_equal(gm.labels().ravel(), g["labels"])


def test_batch_autotune_and_fp32(gpu, tmp_path):
    """FP32+Kahan batch: error against the FP64 oracle per domain."""
    geo = [(64, 64, 64, 50, 40, 21), (50, 72, 60, 80, 30, 22), (80, 50, 50, 30, 60, 23)]
    params, doms = [], []
    for k, (nx, ny, nz, ng, nn, seed) in enumerate(geo):
        params.append(sg.read_uds(sg.UdsSpec(nx=nx, ny=ny, nz=nz, precision=1).write(tmp_path / f"f{k}.uds")))
        doms.append(sg.generate_domain(nx, ny, nz, ng, nn, seed=seed))
    with sg.Batch(params) as b:
        for i, d in enumerate(doms):
            b.load_domain(i, d)
        t = b.autotune()
        assert t.steps > 0
        b.run_until()
        for i, (p, d) in enumerate(zip(params, doms)):
            p64 = sg.Params.from_buffer_copy(p)
            p64.precision = 0
            ref = oracle.run(p64, d)
            lab = b.labels(i).ravel()
            mismatch = float(np.mean(lab != ref["labels"]))
            assert mismatch < 1e-3, f"domain {i}: label mismatch {mismatch}"
            x32 = np.array([s.X for s in b.trace(i)])
            x64 = ref["trace"]["X"]
            m = min(len(x32), len(x64))
            assert np.max(np.abs(x32[:m] - x64[:m])) < 5e-3


def test_phase_timing_is_sampled(gpu, tmp_path):
    """Phase events on every k-th step only; results do not depend on it."""
    p, d, g = load_case("base", tmp_path)
    nsteps = len(g["t"])
    with sg.GrowthMachine(p) as gm:
        gm.load_domain(d)
        for every, expect in ((1, nsteps), (0, 0), (8, (nsteps + 7) // 8)):
            gm.set_tune(timing_every=every)
            gm.restart()
            gm.place_nuclei()
            tr = gm.run_until()
            t = gm.timing()
            assert t.grow_launches == nsteps and t.timed_steps == expect, (every, t.timed_steps)
            assert (t.fill_ms > 0) == (expect > 0) and t.fill_ms <= t.grow_ms
            assert_trace(tr, g, f"timing_every={every}")
