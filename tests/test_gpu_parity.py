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

FIELDS_EXACT = ["Xcells", "Sv", "n_full", "n_new", "t", "dt", "dt_used", "Pmax", "rhomax", "n_nuclei"]


def run_gpu(p, d, ptable=None, x_target=-1.0):
    with sg.GrowthMachine(p, device=0) as gm:
        gm.load_domain(d, ptable)
        gm.place_nuclei()
        tr = gm.run_until(x_target)
        lab = gm.labels()
        rc, dc = gm.grain_counts()
    return tr, lab, rc, dc


def assert_same(tr, lab, rc, dc, ref):
    ot = ref["trace"]
    assert len(tr) == len(ot), f"step count {len(tr)} vs oracle {len(ot)}"
    for f in FIELDS_EXACT:
        g = np.array([getattr(s, f) for s in tr])
        assert np.array_equal(g, ot[f]), f"{f} differs first at step {int(np.argmax(g != ot[f]))}"
    nn = np.array([list(s.next_never) for s in tr])
    assert np.array_equal(nn, ot["next_never"]), "slot high-water marks differ (slot order diverged)"
    nr = np.array([list(s.n_recycled) for s in tr])
    assert np.array_equal(nr, ot["n_recycled"]), "recycle-list lengths differ"
    assert np.array_equal(lab.ravel(), ref["labels"]), "final labels differ"
    assert np.array_equal(rc, ref["rxg_counts"]) and np.array_equal(dc, ref["defg_counts"]), "grain counts differ"


def compare(p, d, ptable=None):
    ref = oracle.run(p, d, ptable)
    assert ref["status"] == 0
    out = run_gpu(p, d, ptable)
    assert_same(*out, ref)
    return out, ref


# odd extents put padding words in the device grid's 2x2x2 bricks
@pytest.mark.parametrize("shape,ngr,nnuc,seed", [((64, 64, 64), 40, 24, 7), ((50, 72, 56), 90, 60, 3), ((45, 51, 37), 60, 40, 5)])
def test_fp64_matches_oracle(gpu, tmp_uds, shape, ngr, nnuc, seed):
    nx, ny, nz = shape
    d = sg.generate_domain(nx, ny, nz, ngr, nnuc, seed=seed)
    compare(sg.read_uds(tmp_uds(sg.UdsSpec(nx=nx, ny=ny, nz=nz))), d)


def test_fp64_distinct_mobilities(gpu, tmp_uds):
    d = sg.generate_domain(64, 64, 64, 60, 40, seed=11)
    compare(sg.read_uds(tmp_uds(sg.UdsSpec(nx=64, ny=64, nz=64, LAGBm0="30.0", GSm0="600.0"))), d)


def test_fp64_rollett_holm(gpu, tmp_uds):
    d = sg.generate_domain(64, 64, 64, 60, 40, seed=12)
    compare(sg.read_uds(tmp_uds(sg.UdsSpec(nx=64, ny=64, nz=64, mobility_model=2))), d)


def test_fp64_defragmentation(gpu, tmp_uds):
    d = sg.generate_domain(64, 64, 64, 50, 30, seed=13)
    spec = sg.UdsSpec(nx=64, ny=64, nz=64, defragmentation=1, defrag_x=["0.2", "0.5", "0.8"])
    compare(sg.read_uds(tmp_uds(spec)), d)


def test_fp64_periodic_boundary(gpu, tmp_uds):
    d = sg.generate_domain(56, 64, 60, 50, 30, seed=14)
    compare(sg.read_uds(tmp_uds(sg.UdsSpec(nx=56, ny=64, nz=60, boundary=1))), d)


def test_fp64_periodic_boundary_odd_extents(gpu, tmp_uds):
    """Periodic wrap across the padded last brick of every axis."""
    d = sg.generate_domain(33, 47, 29, 30, 20, seed=16)
    compare(sg.read_uds(tmp_uds(sg.UdsSpec(nx=33, ny=47, nz=29, boundary=1))), d)


def test_fp64_border_grow_policy(gpu, tmp_uds):
    d = sg.generate_domain(64, 64, 64, 50, 200, seed=15)
    compare(sg.read_uds(tmp_uds(sg.UdsSpec(nx=64, ny=64, nz=64, border_policy=1, initial_cache="0.05"))), d)


def test_fp64_incubation_times(gpu, tmp_uds):
    d = sg.generate_domain(64, 64, 64, 50, 60, seed=16, nucleation_rate=3000.0)
    assert d.rxg_tincub.max() > 0
    compare(sg.read_uds(tmp_uds(sg.UdsSpec(nx=64, ny=64, nz=64))), d)


def test_fp64_incubation_repeated_and_face_sites(gpu, tmp_uds):
    """Nuclei due during the run are placed on the device: repeated sites (the later nucleus
    is not placed), sites on the faces (Border list), and steps that defragment (placed by
    the host) must all give the oracle's slots, counts and labels."""
    d = sg.generate_domain(64, 64, 64, 50, 400, seed=21, nucleation_rate=2000.0)
    site = d.rxg_site.copy()
    site[1::7] = site[0::7][: len(site[1::7])]
    k = np.arange(0, len(site), 11)
    x, y, z = site[k] % 64, (site[k] // 64) % 64, site[k] // 4096
    x[::2] = 0
    z[1::2] = 63
    site[k] = (z * 64 + y) * 64 + x
    d2 = sg.Domain(d.nx, d.ny, d.nz, d.grid, d.defg_quat, d.defg_rho0, d.rxg_quat, site.astype(np.uint32), d.rxg_tincub)
    (tr, *_), _ = compare(sg.read_uds(tmp_uds(sg.UdsSpec(nx=64, ny=64, nz=64))), d2)
    assert sum(s.n_nuclei for s in tr) < len(site)  # some were not placeable
    spec = sg.UdsSpec(nx=64, ny=64, nz=64, defragmentation=1, defrag_x=["0.1", "0.3", "0.6"])
    compare(sg.read_uds(tmp_uds(spec)), d2)


def test_fp64_recovery_refreshes_velocities(gpu, tmp_uds):
    d = sg.generate_domain(64, 64, 64, 50, 30, seed=17)
    compare(sg.read_uds(tmp_uds(sg.UdsSpec(nx=64, ny=64, nz=64, recovery=10, recovery_k="20.0"))), d)
    compare(sg.read_uds(tmp_uds(sg.UdsSpec(nx=64, ny=64, nz=64, recovery=3))), d)


def test_fp64_recovery_refresh_mixes(gpu, tmp_uds):
    """Recovery refreshes every velocity factor every step from the cached mobilities:
    Rollett-Holm, distinct LAGB / GS mobilities, and a heating schedule that interleaves full
    refreshes from the P table (new mobilities) with the cached-mobility refreshes."""
    d = sg.generate_domain(64, 64, 64, 60, 40, seed=22)
    compare(sg.read_uds(tmp_uds(sg.UdsSpec(nx=64, ny=64, nz=64, recovery=10, recovery_k="20.0", mobility_model=2))), d)
    compare(sg.read_uds(tmp_uds(sg.UdsSpec(nx=64, ny=64, nz=64, recovery=10, recovery_k="20.0", LAGBm0="30.0", GSm0="600.0"))), d)
    spec = sg.UdsSpec(nx=64, ny=64, nz=64, recovery=10, recovery_k="20.0",
                      schedule=[("0.0", "700.0"), ("0.05", "760.0"), ("360000.0", "760.0")])
    compare(sg.read_uds(tmp_uds(spec)), d)


def test_fp64_heating_schedule(gpu, tmp_uds):
    d = sg.generate_domain(64, 64, 64, 50, 30, seed=18)
    spec = sg.UdsSpec(nx=64, ny=64, nz=64, schedule=[("0.0", "700.0"), ("0.05", "760.0"), ("360000.0", "760.0")])
    compare(sg.read_uds(tmp_uds(spec)), d)


def test_fp64_zener_drag(gpu, tmp_uds):
    d = sg.generate_domain(64, 64, 64, 50, 30, seed=19)
    compare(sg.read_uds(tmp_uds(sg.UdsSpec(nx=64, ny=64, nz=64, zener=1, zener_table=[("0.0", "2.0e5"), ("360000.0", "2.0e5")]))), d)


def test_fp64_user_ptable(gpu, tmp_uds):
    d = sg.generate_domain(60, 60, 60, 40, 25, seed=20)
    p = sg.read_uds(tmp_uds(sg.UdsSpec(nx=60, ny=60, nz=60, LAGBm0="30.0", GSm0="600.0")))
    pt = np.array([[sg.mobility_weight(p, d.rxg_quat[r], d.defg_quat[g]) for g in range(d.ndefg)] for r in range(d.nrxg)])
    compare(p, d, pt)


def test_restart_and_reload_reproduce(gpu, tmp_uds):
    d = sg.generate_domain(64, 64, 64, 40, 24, seed=21)
    p = sg.read_uds(tmp_uds(sg.UdsSpec(nx=64, ny=64, nz=64)))
    ref = oracle.run(p, d)
    with sg.GrowthMachine(p, device=0) as gm:
        gm.load_domain(d)
        for _ in range(2):
            gm.place_nuclei()
            tr = gm.run_until()
            lab = gm.labels()
            rc, dc = gm.grain_counts()
            assert_same(tr, lab, rc, dc, ref)
            gm.restart()
        d2 = sg.generate_domain(64, 64, 64, 40, 24, seed=22)
        ref2 = oracle.run(p, d2)
        gm.load_domain(d2)
        gm.place_nuclei()
        tr = gm.run_until()
        assert_same(tr, gm.labels(), *gm.grain_counts(), ref2)


def test_fp32_kahan_error_is_small(gpu, tmp_uds):
    """FP32+Kahan fill vs the FP64 oracle: label mismatch, max |dX(t)|, mean grain size error."""
    d = sg.generate_domain(96, 96, 96, 120, 80, seed=23)
    p64 = sg.read_uds(tmp_uds(sg.UdsSpec(nx=96, ny=96, nz=96)))
    p32 = sg.read_uds(tmp_uds(sg.UdsSpec(nx=96, ny=96, nz=96, precision=1)))
    ref = oracle.run(p64, d)
    tr, lab, rc, dc = run_gpu(p32, d)
    mismatch = np.mean(lab.ravel() != ref["labels"])
    x32 = np.array([s.X for s in tr])
    x64 = ref["trace"]["X"]
    n = min(len(x32), len(x64))
    dx = np.max(np.abs(x32[:n] - x64[:n]))
    gs_err = abs(rc.mean() - ref["rxg_counts"].mean()) / ref["rxg_counts"].mean()
    assert mismatch < 1e-3, mismatch
    assert dx < 5e-3, dx
    assert gs_err < 1e-3, gs_err


# ---------------------------------------------------------------- against the reference's own outputs
from _golden import TRACE_FIELDS, first_difference, growth_cases, load_case  # noqa: E402


@pytest.mark.parametrize("name", growth_cases())
def test_gpu_reproduces_reference_golden(gpu, tmp_path, name):
    """The sm_103a path against the fixtures the reference's growth loop produced."""
    p, d, g = load_case(name, tmp_path)
    tr, lab, rc, dc = run_gpu(p, d)
    for f in TRACE_FIELDS:
        a = np.array([getattr(s, f) for s in tr])
        assert np.array_equal(a, g[f]), f"{f}: {first_difference(a, g[f])}"
    assert np.array_equal(lab.ravel(), g["labels"]), "final labels"
    assert np.array_equal(rc, g["rxg_counts"]) and np.array_equal(dc, g["defg_counts"])


# ---------------------------------------------------------------- the benchmark configurations
from _golden import config_cases, labels_digest, load_config  # noqa: E402


@pytest.mark.parametrize("name", ["config0_128", pytest.param("config1_512", marks=pytest.mark.slow)])
def test_gpu_reproduces_reference_at_benchmark_size(gpu, tmp_path, name):
    """The benchmark configurations at their full sizes against the reference's own run of
    them: config 0 (128^3, 500 grains, 200 nuclei) and config 1, the headline workload's
    512^3 domain (20,000 grains, 50,000 nuclei).  Every step's t, dt, X cells, Sv, full
    cells, P max and rho max, the final labels (SHA-256 of all N labels) and every grain's
    cell count, bit for bit."""
    assert name in config_cases()
    p, d, g = load_config(name, tmp_path)
    tr, lab, rc, dc = run_gpu(p, d)
    for f in TRACE_FIELDS:
        a = np.array([getattr(s, f) for s in tr])
        assert np.array_equal(a, g[f]), f"{f}: {first_difference(a, g[f])}"
    assert labels_digest(lab) == g["labels_sha256"], "final labels"
    assert np.array_equal(rc, g["rxg_counts"]) and np.array_equal(dc, g["defg_counts"])
