"""On-the-fly characterization and ensemble post-processing, CPU side: the oracle against the
reference's own grain-evolution log (log_grainevo, log_rxareaprofile at the SingleGrainVolOverTime
logpoints, SCORE_OnTheFlyCharacterization.cpp:274-384, 478-531), its get_interpCellCount
(SCORE_SolitaryUnitAveraging.cpp:1304-1365) and the ensemble sums of postprocess_rediscr_kinetics /
postprocess_rediscr_macrotexture formed from the reference's values in the reference's order.
Everything here is compared bit for bit."""
import numpy as np

import oracle
from _golden import evo_descriptor, load_evolution


def test_oracle_grain_evolution_log_matches_reference(built, tmp_path):
    doms, _ = load_evolution(tmp_path)
    for p, d, g in doms:
        assert p.n_logpoints == 10 and p.rxarea_threshold == 13
        sim = oracle.Sim(p, d)
        assert sim.advance()["status"] == 0
        assert sim.time() == g["t_end"]
        log = sim.grainevo(d.nz)
        sim.close()
        assert len(log) == len(g["snap_t"]) == 10
        for i, s in enumerate(log):
            assert s["t"] == g["snap_t"][i] and s["X"] == g["snap_X"][i], i
            assert s["step"] == g["snap_step"][i] and s["Sv"] == g["snap_Sv"][i], i
            assert np.array_equal(s["counts"], g["snap_counts"][i]), i
            assert np.array_equal(s["area"], g["areas"][i]), i
        # the profile is not trivial: rx sections below the threshold are left out somewhere
        assert any(a[:, 0].sum() < (s["counts"][d.ndefg:]).sum() for a, s in zip(g["areas"], log))


def test_oracle_interpolation_matches_reference(built, tmp_path):
    doms, ens = load_evolution(tmp_path)
    n = ens["nslots"]
    dt = ens["tmax"] / (n - 1)
    times = [0.0 + (k + 1) * dt for k in range(n)]
    assert times[-1] > ens["tmax"]  # the last slot lies past the end, as the reference's scheme has it
    for p, d, g in doms:
        desc = evo_descriptor(d, g)
        got = np.array([[oracle.interp_count(desc, gid, w) for gid in range(d.ndefg + d.nrxg)] for w in times])
        assert np.array_equal(got, g["interp"])


def test_oracle_rediscretization_matches_reference(built, tmp_path):
    doms, ens = load_evolution(tmp_path)
    descs = [evo_descriptor(d, g) for _, d, g in doms]
    t, vol, box = oracle.rediscr_kinetics(descs, ens["nslots"])
    assert box == float(sum(d.ncells for _, d, _ in doms))
    assert np.array_equal(vol, ens["kinetics"])
    assert 0.0 < vol[0] / box < vol[-1] / box <= 1.0
    t2, tex = oracle.rediscr_texture(descs, ens["nslots"], ens["nclass"])
    assert np.array_equal(t, t2) and np.array_equal(tex, ens["texture"])
