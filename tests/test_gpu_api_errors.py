"""Error behaviour of the C ABI on a GPU: calls out of sequence, inconsistent inputs and
exhausted resources return a status (never abort), leave the context usable where the
header says so, and leave no pending CUDA error behind for other users of the device."""
import ctypes as C

import numpy as np
import pytest

import score_gb300 as sg
from score_gb300 import _abi

pytestmark = pytest.mark.gpu


def small_params(tmp_path, **kw):
    return sg.read_uds(sg.UdsSpec(nx=50, ny=50, nz=50, **kw).write(tmp_path / "p.uds"))


def test_calls_out_of_sequence(gpu, tmp_path):
    lib = _abi.load()
    p = small_params(tmp_path)
    ctx = C.c_void_p()
    assert lib.score_create(C.byref(ctx), C.byref(p), 0) == _abi.OK
    try:
        st = _abi.StepStats()
        assert lib.score_step(ctx, C.byref(st)) == _abi.ERR_STATE
        assert lib.score_place_nuclei(ctx, None) == _abi.ERR_STATE
        lab = np.empty(50 ** 3, dtype=np.uint32)
        assert lib.score_export_labels(ctx, lab.ctypes.data) == _abi.ERR_STATE
        assert lib.score_restart(ctx) == _abi.ERR_STATE
        assert b"no domain" in lib.score_last_error(ctx)
    finally:
        lib.score_destroy(ctx)


def test_inconsistent_domains_are_refused(gpu, tmp_path):
    p = small_params(tmp_path)
    d = sg.generate_domain(50, 50, 50, 10, 5, seed=1)
    with sg.GrowthMachine(p) as gm:
        bad_site = sg.Domain(50, 50, 50, d.grid, d.defg_quat, d.defg_rho0, d.rxg_quat,
                             np.array([0, 1, 2, 3, 50 ** 3], dtype=np.uint32), d.rxg_tincub)
        with pytest.raises(sg.ScoreError) as e:
            gm.load_domain(bad_site)
        assert e.value.status == _abi.ERR_ARG
        bad_grid = d.grid.copy()
        bad_grid[3, 4, 5] = 10  # only ids 0..9 exist
        with pytest.raises(sg.ScoreError) as e:
            gm.load_domain(sg.Domain(50, 50, 50, bad_grid, d.defg_quat, d.defg_rho0, d.rxg_quat, d.rxg_site, d.rxg_tincub))
        assert e.value.status == _abi.ERR_ARG
        # the context still works with a good domain
        gm.load_domain(d)
        gm.place_nuclei()
        tr = gm.run_until()
        assert tr and tr[-1].X > 0.99


def test_tune_values_are_checked(gpu, tmp_path):
    with sg.GrowthMachine(small_params(tmp_path)) as gm:
        with pytest.raises(sg.ScoreError):
            gm.set_tune(items=5)
        with pytest.raises(sg.ScoreError):
            gm.set_tune(fill_blocks_per_sm=0)
        with pytest.raises(sg.ScoreError):
            gm.set_tune(spec_holes_pct=101)
        assert gm.tune().spec_holes_pct == 30
        gm.set_tune(items=16, use_graph=0, spec_holes_pct=0)
        t = gm.tune()
        assert t.items == 16 and t.use_graph == 0 and t.spec_holes_pct == 0


def test_batch_limits(gpu, tmp_path):
    lib = _abi.load()
    p64 = small_params(tmp_path)
    p32 = small_params(tmp_path, precision=1)
    b = C.c_void_p()
    mixed = (_abi.Params * 2)(p64, p32)
    assert lib.score_batch_create(C.byref(b), mixed, 2, 0) == _abi.ERR_ARG  # one precision per batch
    many = (_abi.Params * 65)(*([p64] * 65))
    assert lib.score_batch_create(C.byref(b), many, 65, 0) == _abi.ERR_ARG  # at most 64 domains
    # the device's 64 argument slots: a full batch leaves none for another context
    with sg.Batch([p64] * 64) as full:
        ctx = C.c_void_p()
        assert lib.score_create(C.byref(ctx), C.byref(p64), 0) == _abi.ERR_CAPACITY
        assert not ctx.value
        assert len(full) == 64
    with sg.GrowthMachine(p64):  # slots are returned when the batch closes
        pass


def test_no_pending_cuda_error_is_left_behind(gpu, tmp_path):
    import torch
    p = small_params(tmp_path)
    d = sg.generate_domain(50, 50, 50, 10, 5, seed=2)
    with sg.GrowthMachine(p) as gm:
        gm.load_domain(d)
        gm.place_nuclei()
        gm.run_until()
        gm.set_tune(use_graph=0)
        gm.restart()
        gm.place_nuclei()
        gm.run_until()
    x = torch.ones(4, device="cuda")  # raises if the library left an error in the runtime
    assert float(x.sum()) == 4.0
