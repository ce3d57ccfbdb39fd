"""score_mobility_table_noalloc: the device FP64 mobility-weight table that allocates
no device memory, checked against the host entry point score_mobility_weight.

Two calls in a row (different sizes, different data, different mobility models)
must each match the host within the tolerance below and return the table's maximum:
the second call only gets its maximum if the first one left the static scratch's
completion counter at zero.  A repeat of the first call must reproduce it bit for
bit, and a table with more rows than the static scratch holds is refused before any
launch.  Buffers of the test itself come from torch; the entry point allocates none.
"""
import ctypes as C

import numpy as np
import pytest

import score_gb300 as sg
from score_gb300 import _abi

pytestmark = pytest.mark.gpu

# CUDA's acos/cos/exp/pow against glibc's: a few ulp of P in [-1, 1]
ATOL = 1e-12
MAX_ROWS = 65536
ERR_SCRATCH_LIMIT = -11


def _unit(q):
    return q / np.linalg.norm(q, axis=-1, keepdims=True)


def _qmul(a, b):
    a0, a1, a2, a3 = np.moveaxis(a, -1, 0)
    b0, b1, b2, b3 = np.moveaxis(b, -1, 0)
    return np.stack([a0 * b0 - a1 * b1 - a2 * b2 - a3 * b3,
                     a0 * b1 + a1 * b0 + a2 * b3 - a3 * b2,
                     a0 * b2 - a1 * b3 + a2 * b0 + a3 * b1,
                     a0 * b3 + a1 * b2 - a2 * b1 + a3 * b0], axis=-1)


def _axis_angle(axis, deg):
    axis = np.asarray(axis, dtype=np.float64)
    axis = axis / np.linalg.norm(axis, axis=-1, keepdims=True)
    h = np.radians(deg) / 2.0
    return np.concatenate([np.cos(h)[..., None], np.sin(h)[..., None] * axis], axis=-1)


def orientations(seed, nrxg, ndefg):
    """Deformed grains uniform; recrystallized grains a mix of uniform orientations,
    small rotations of a deformed grain (LAGB, P = -1) and rotations near 40deg<111>
    (the cos^2 branch), so every branch of the weight is exercised."""
    rng = np.random.default_rng(seed)
    qd = _unit(rng.normal(size=(ndefg, 4)))
    qr = _unit(rng.normal(size=(nrxg, 4)))
    k = nrxg // 3
    src = rng.integers(0, ndefg, size=2 * k)
    small = _axis_angle(rng.normal(size=(k, 3)), rng.uniform(1.0, 12.0, size=k))
    qr[:k] = _qmul(qd[src[:k]], small)
    near = _axis_angle(np.ones((k, 3)) + rng.normal(scale=0.03, size=(k, 3)), 40.0 + rng.uniform(-4.0, 4.0, size=k))
    qr[k:2 * k] = _qmul(qd[src[k:]], near)
    return np.ascontiguousarray(_unit(qr)), np.ascontiguousarray(qd)


def host_table(p, qr, qd):
    return np.array([[sg.mobility_weight(p, qr[i], qd[j]) for j in range(len(qd))] for i in range(len(qr))])


def device_table(lib, p, qr, qd):
    import torch
    dev = torch.device("cuda:0")
    d_qr = torch.from_numpy(qr).to(dev)
    d_qd = torch.from_numpy(qd).to(dev)
    d_tab = torch.full((len(qr), len(qd)), float("nan"), dtype=torch.float64, device=dev)
    d_pmax = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = lib.score_mobility_table_noalloc(C.byref(p), d_qr.data_ptr(), len(qr), d_qd.data_ptr(), len(qd),
                                          d_tab.data_ptr(), d_pmax.data_ptr(), C.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.score_status_string(rc).decode()
    stream.synchronize()
    return d_tab.cpu().numpy(), float(d_pmax.cpu().item())


def rh_params():
    p = sg.default_params()
    p.mobility_model = 2
    p.RH_cut, p.RH_trans, p.RH_exponent = 0.99, 5.0, 4.0
    return p


def test_table_two_calls_match_host(gpu):
    import torch
    torch.cuda.set_device(0)
    lib = _abi.load()
    cases = [(sg.default_params(), orientations(11, 37, 301)), (rh_params(), orientations(12, 64, 129))]
    first = None
    for p, (qr, qd) in cases:
        tab, pmax = device_table(lib, p, qr, qd)
        ref = host_table(p, qr, qd)
        assert np.isfinite(tab).all(), "entries left unwritten"
        err = np.abs(tab - ref)
        assert err.max() <= ATOL, f"max |P_device - P_host| = {err.max():.3e} at {np.unravel_index(err.argmax(), err.shape)}"
        assert abs(pmax - ref.max()) <= ATOL, f"table max {pmax!r} vs host {ref.max()!r}"
        if first is None:
            first = tab
            # all three classes of the Sebald-Gottstein weight occur
            assert (ref == -1.0).any() and (ref == 0.0).any() and ((ref > 0.0) & (ref < 1.0)).any()
    # the same inputs again: the same bits
    p, (qr, qd) = cases[0]
    again, _ = device_table(lib, p, qr, qd)
    assert np.array_equal(again.view(np.uint64), first.view(np.uint64))


def test_table_rejects_more_rows_than_scratch(gpu):
    import torch
    lib = _abi.load()
    dev = torch.device("cuda:0")
    one = torch.zeros(4, dtype=torch.float64, device=dev)
    rc = lib.score_mobility_table_noalloc(C.byref(sg.default_params()), one.data_ptr(), MAX_ROWS + 1, one.data_ptr(), 1,
                                          one.data_ptr(), one.data_ptr(), None)
    assert rc == ERR_SCRATCH_LIMIT
    assert b"scratch" in lib.score_status_string(rc)
    # and the scratch is still usable afterwards
    qr, qd = orientations(13, 5, 7)
    tab, pmax = device_table(lib, sg.default_params(), qr, qd)
    ref = host_table(sg.default_params(), qr, qd)
    assert np.abs(tab - ref).max() <= ATOL and abs(pmax - ref.max()) <= ATOL
