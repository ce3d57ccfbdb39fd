"""On-the-fly characterization and ensemble post-processing on the GPU, bit for bit against the
reference's grain-evolution log (log_grainevo + log_rxareaprofile at the SingleGrainVolOverTime
logpoints) and the ensemble sums made from its get_interpCellCount values, and, at a larger size,
against the oracle."""
import numpy as np
import pytest

import oracle
import score_gb300 as sg
from _golden import evo_descriptor, load_evolution

pytestmark = pytest.mark.gpu


def assert_log(log, ref, ndefg):
    assert len(log) == len(ref["snap_t"])
    for i, (info, cnt, area) in enumerate(log):
        assert info.t == ref["snap_t"][i] and info.X == ref["snap_X"][i], i
        assert info.step == ref["snap_step"][i] and info.Sv == ref["snap_Sv"][i], i
        assert np.array_equal(cnt, ref["snap_counts"][i]), f"counts of snapshot {i}"
        assert np.array_equal(area, ref["areas"][i]), f"RX area profile of snapshot {i}"


def test_gpu_grain_evolution_log_matches_reference(gpu, tmp_path):
    doms, _ = load_evolution(tmp_path)
    for p, d, g in doms:
        with sg.GrowthMachine(p, device=0) as gm:
            gm.load_domain(d)
            for _ in range(2):  # a restart clears the log and takes it again
                gm.place_nuclei()
                gm.run_until()
                assert_log(gm.grainevo(), g, d.ndefg)
                gm.restart()


def test_gpu_ensemble_postprocessing_matches_reference(gpu, tmp_path):
    doms, ens = load_evolution(tmp_path)
    with sg.Batch([p for p, _, _ in doms], device=0) as b:
        for k, (_, d, _) in enumerate(doms):
            b.load_domain(k, d)
        b.place_nuclei()
        b.run_until()
        for k, (_, d, g) in enumerate(doms):
            assert_log(b.grainevo(k), g, d.ndefg)
        t, vol, box = b.rediscr_kinetics(ens["nslots"])
        assert box == float(sum(d.ncells for _, d, _ in doms))
        assert np.array_equal(vol, ens["kinetics"]), "rediscretized kinetics"
        cls = np.concatenate([g["cls"] for _, _, g in doms])
        t2, tex = b.rediscr_texture(ens["nslots"], cls, ens["nclass"])
        assert np.array_equal(t, t2)
        assert np.array_equal(tex, ens["texture"]), "rediscretized macrotexture"
        sizes = b.final_grain_sizes()
        assert np.array_equal(sizes, np.concatenate([g["final"][d.ndefg:] for _, d, g in doms]))


def test_gpu_grain_evolution_at_128_matches_oracle(gpu, tmp_path):
    """The 128^3 benchmark configuration with eleven logpoints and an RX area threshold of 5: every
    snapshot and profile of the GPU run equals the oracle's; its rediscretized kinetics (an ensemble
    of one) equals the oracle's post-processing of the same log."""
    d = sg.generate_domain(128, 128, 128, 500, 200, seed=0)
    spec = sg.UdsSpec(nx=128, ny=128, nz=128, logpoints=["0.0"] + [f"{x / 10:.1f}" for x in range(1, 10)] + ["0.95"],
                      area_threshold=5)
    p = sg.read_uds(spec.write(tmp_path / "c0.uds"))
    sim = oracle.Sim(p, d)
    sim.advance()
    ref = sim.grainevo(d.nz)
    fin = sim.finish()
    t_end = sim.time()
    sim.close()
    with sg.GrowthMachine(p, device=0) as gm:
        gm.load_domain(d)
        gm.place_nuclei()
        gm.run_until()
        log = gm.grainevo()
        t, vol, box = gm.rediscr_kinetics(100)
    assert len(log) == len(ref) == 11
    for (info, cnt, area), r in zip(log, ref):
        assert (info.t, info.X, info.step, info.Sv) == (r["t"], r["X"], r["step"], r["Sv"])
        assert np.array_equal(cnt, r["counts"]) and np.array_equal(area, r["area"])
    desc = {"ndefg": d.ndefg, "nrxg": d.nrxg, "t": np.array([r["t"] for r in ref]), "counts": np.array([r["counts"] for r in ref]),
            "final": np.concatenate([fin["defg_counts"], fin["rxg_counts"]]), "tsimend": t_end, "cells": d.ncells}
    t_o, vol_o, box_o = oracle.rediscr_kinetics([desc], 100)
    assert np.array_equal(t, t_o) and np.array_equal(vol, vol_o) and box == box_o


def test_gpu_grain_evolution_odd_extents_matches_oracle(gpu, tmp_path):
    """Odd extents (padding words in the device grid's bricks): snapshots and RX area profiles."""
    d = sg.generate_domain(45, 51, 37, 60, 40, seed=5)
    spec = sg.UdsSpec(nx=45, ny=51, nz=37, logpoints=["0.0", "0.3", "0.6", "0.9"], area_threshold=3)
    p = sg.read_uds(spec.write(tmp_path / "odd.uds"))
    sim = oracle.Sim(p, d)
    sim.advance()
    ref = sim.grainevo(d.nz)
    sim.close()
    with sg.GrowthMachine(p, device=0) as gm:
        gm.load_domain(d)
        gm.place_nuclei()
        gm.run_until()
        log = gm.grainevo()
    assert len(log) == len(ref) == 4
    for (info, cnt, area), r in zip(log, ref):
        assert (info.t, info.X, info.step, info.Sv) == (r["t"], r["X"], r["step"], r["Sv"])
        assert np.array_equal(cnt, r["counts"]) and np.array_equal(area, r["area"])
