"""GPU parity: the sm_103a growth path against the CPU oracle, bit for bit (FP64).

Compared per step: Xcells (X(t)), Sv, full-cell count, t, dt, P max, rho max,
the slot high-water marks and recycle lengths (slot order), and at the end the
final grain labels and per-grain cell counts.  Integer and index results must be
identical; FP64 results must be identical too (the path is bit-exact by design).
"""
import numpy as np
import pytest

import oracle
import score_gb300 as sg

pytestmark = pytest.mark.gpu

FIELDS_EXACT = ["Xcells", "Sv", "n_full", "t", "dt", "dt_used", "Pmax", "rhomax"]


def run_gpu(p, d, ptable=None, x_target=-1.0):
    with sg.GrowthMachine(p, device=0) as gm:
        gm.load_domain(d, ptable)
        gm.place_nuclei()
        tr = gm.run_until(x_target)
        lab = gm.labels()
        rc, dc = gm.grain_counts()
        tm = gm.timing()
    return tr, lab, rc, dc, tm


def compare(p, d, ptable=None):
    ref = oracle.run(p, d, ptable)
    assert ref["status"] == 0
    tr, lab, rc, dc, _ = run_gpu(p, d, ptable)
    ot = ref["trace"]
    assert len(tr) == len(ot), f"step count {len(tr)} vs oracle {len(ot)}"
    for f in FIELDS_EXACT:
        g = np.array([getattr(s, f) for s in tr])
        assert np.array_equal(g, ot[f]), f"{f} differs at step {int(np.argmax(g != ot[f]))}"
    nn = np.array([list(s.next_never) for s in tr])
    assert np.array_equal(nn, ot["next_never"]), "slot high-water marks differ (slot order diverged)"
    nr = np.array([list(s.n_recycled) for s in tr])
    assert np.array_equal(nr, ot["n_recycled"]), "recycle-list lengths differ"
    assert np.array_equal(lab.ravel(), ref["labels"]), "final labels differ"
    assert np.array_equal(rc, ref["rxg_counts"]) and np.array_equal(dc, ref["defg_counts"])
    return tr, ref


@pytest.mark.parametrize("shape,ngr,nnuc,seed", [((64, 64, 64), 40, 24, 7), ((50, 72, 56), 90, 60, 3)])
def test_fp64_matches_oracle(gpu, tmp_uds, shape, ngr, nnuc, seed):
    nx, ny, nz = shape
    d = sg.generate_domain(nx, ny, nz, ngr, nnuc, seed=seed)
    p = sg.read_uds(tmp_uds(sg.UdsSpec(nx=nx, ny=ny, nz=nz)))
    compare(p, d)


def test_fp64_distinct_mobilities_matches_oracle(gpu, tmp_uds):
    d = sg.generate_domain(64, 64, 64, 60, 40, seed=11)
    spec = sg.UdsSpec(nx=64, ny=64, nz=64, LAGBm0="30.0", GSm0="600.0")
    compare(sg.read_uds(tmp_uds(spec)), d)


def test_fp64_rollett_holm_matches_oracle(gpu, tmp_uds):
    d = sg.generate_domain(64, 64, 64, 60, 40, seed=12)
    spec = sg.UdsSpec(nx=64, ny=64, nz=64, mobility_model=2, RH_HAGBHact="2.45")
    compare(sg.read_uds(tmp_uds(spec)), d)
