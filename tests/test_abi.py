"""The C ABI library without a GPU: it loads, exports every function that
include/score_gb300.h declares, and its host-side logic (status strings, .uds
parsing, parameter validation, deterministic generator) behaves as specified.
No call here launches device work."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import score_gb300 as sg
from score_gb300 import _abi

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "score_gb300.h"


def declared_functions() -> set[str]:
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return set(re.findall(r"^\s*(?:int|void|const char\s*\*)\s+(score_\w+)\s*\(", text, flags=re.M))


def test_library_exports_every_declared_function(built):
    lib = _abi.load()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"
    assert names == set(_abi.SIGNATURES), "ctypes signature table and header disagree"


def test_library_is_the_in_tree_build(built):
    path = Path(_abi.load()._name).resolve()
    assert path.is_relative_to(ROOT), path


def test_status_strings(built):
    lib = _abi.load()
    assert lib.score_abi_version() == 4
    assert lib.score_status_string(0) == b"ok"
    for code in range(-1, -12, -1):
        s = lib.score_status_string(code)
        assert s and s != b"unknown status", code
    assert lib.score_status_string(-999) == b"unknown status"


def test_uds_roundtrip(built, tmp_uds):
    spec = sg.UdsSpec(nx=64, ny=72, nz=80, cellsize_um="2.5", maxfill="0.05", mobility_model=2, RH_exponent="7.5",
                      schedule=[("0.0", "600.0"), ("10.0", "700.0"), ("360000.0", "700.0")], recovery=10, recovery_k="0.5",
                      boundary=1, precision=1, border_policy=1)
    p = sg.read_uds(tmp_uds(spec))
    assert (p.nx, p.ny, p.nz) == (64, 72, 80)
    assert p.cellsize == 2.5 * 1e-6
    assert p.maxfillperstep == 0.05
    assert p.mobility_model == 2 and p.RH_exponent == 7.5
    # temperatures in K; table columns keep the reference's float truncation
    assert p.n_schedule == 3
    assert p.sched_temp[1] == float(np.float32(700.0)) + 273.15
    assert p.sched_time[1] == float(np.float32(10.0))
    # activation enthalpies in J
    assert p.HAGBHact == 2.45 * 1.602176565e-19
    assert p.recovery_model == 10 and p.recovery_k == 0.5
    assert (p.boundary, p.precision, p.border_policy) == (1, 1, 1)


def test_uds_missing_file_is_an_io_error(built, tmp_path):
    with pytest.raises(sg.ScoreError) as e:
        sg.read_uds(tmp_path / "nope.uds")
    assert e.value.status == _abi.ERR_IO


def test_create_validates_before_touching_a_device(built):
    lib = _abi.load()
    ctx = C.c_void_p()
    p = sg.default_params()
    p.nx = p.ny = p.nz = 2  # too small
    assert lib.score_create(C.byref(ctx), C.byref(p), 0) == _abi.ERR_ARG
    assert not ctx.value
    assert lib.score_create(None, C.byref(p), 0) == _abi.ERR_ARG


def test_noalloc_table_rejects_oversize_without_a_device(built):
    lib = _abi.load()
    p = sg.default_params()
    buf = (C.c_double * 4)()
    rc = lib.score_mobility_table_noalloc(C.byref(p), C.addressof(buf), 65537, C.addressof(buf), 1, C.addressof(buf),
                                          C.addressof(buf), None)
    assert rc == -11
    assert lib.score_mobility_table_noalloc(None, None, 1, None, 1, None, None, None) == _abi.ERR_ARG


def test_generator_is_deterministic_and_well_formed(built):
    a = sg.generate_domain(50, 40, 30, 25, 20, seed=5)
    b = sg.generate_domain(50, 40, 30, 25, 20, seed=5)
    c = sg.generate_domain(50, 40, 30, 25, 20, seed=6)
    for f in ("grid", "defg_quat", "defg_rho0", "rxg_quat", "rxg_site", "rxg_tincub"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    assert not np.array_equal(a.grid, c.grid)
    assert a.grid.shape == (30, 40, 50) and a.grid.max() < 25 and len(np.unique(a.grid)) == 25
    assert np.allclose(np.linalg.norm(a.defg_quat, axis=1), 1.0) and np.allclose(np.linalg.norm(a.rxg_quat, axis=1), 1.0)
    assert len(np.unique(a.rxg_site)) == 20 and a.rxg_site.max() < a.ncells
    assert (a.rxg_tincub == 0.0).all()
    r = sg.generate_domain(50, 50, 50, 10, 300, seed=1, nucleation_rate=1000.0)
    assert (np.diff(np.sort(r.rxg_tincub)) >= 0).all() and r.rxg_tincub.max() > 0.0


def test_generator_options(built):
    p = sg.generate_domain(64, 64, 64, 30, 40, seed=2, aspect=(1.0, 4.0, 8.0), ori_mode=1, ncomp=3, scatter_deg=10.0,
                           rho_mode=1, rho_lo=1e14, rho_hi=5e15, site_mode=1, gb_fraction=1.0)
    assert set(np.unique(p.defg_rho0)) <= {1e14, 5e15}
    # every nucleus forced onto a grain boundary: some Moore neighbour has another deformed id
    g = p.grid
    z, rem = np.divmod(p.rxg_site.astype(np.int64), 64 * 64)
    y, x = np.divmod(rem, 64)
    on_gb = np.zeros(len(x), dtype=bool)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                on_gb |= g[(z + dz) % 64, (y + dy) % 64, (x + dx) % 64] != g[z, y, x]
    assert on_gb.all()


# sha256 (first 32 hex digits) of the generator's output arrays; the generator uses
# only integer and correctly rounded arithmetic, so x86-64 and aarch64 hosts agree
GENERATOR_HASHES = [
    (((50, 40, 30, 25, 20, 5), {}), "61eb1305bc48649a625b9bc5c5391eb9"),
    (((64, 64, 64, 30, 40, 2), dict(aspect=(1.0, 4.0, 8.0), ori_mode=1, ncomp=3, scatter_deg=10.0, rho_mode=1, rho_lo=1e14,
                                    rho_hi=5e15, site_mode=1, gb_fraction=1.0)), "68a1c167c597a468608b543ae8ab6173"),
    (((50, 50, 50, 10, 300, 1), dict(nucleation_rate=1000.0)), "2cfe620d71e8addfeb8b1b45dbd9a8df"),
]


@pytest.mark.parametrize("args,kw,digest", [(a, k, h) for (a, k), h in GENERATOR_HASHES])
def test_generator_bits_are_pinned(built, args, kw, digest):
    import hashlib
    d = sg.generate_domain(*args[:5], seed=args[5], **kw)
    h = hashlib.sha256()
    for f in ("grid", "defg_quat", "defg_rho0", "rxg_quat", "rxg_site", "rxg_tincub"):
        h.update(np.ascontiguousarray(getattr(d, f)).tobytes())
    assert h.hexdigest()[:32] == digest
