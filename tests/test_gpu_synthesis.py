"""Deformed-structure synthesis on the GPU (score_generate_domain_gpu): the Voronoi label fill on
the device gives bit for bit the host generator's domain, isotropic and anisotropic, uniform and
grain-boundary nuclei, and the full 512^3 headline domain (its input digest is the one the
reference-made fixture stores)."""
import numpy as np
import pytest

import score_gb300 as sg
from _golden import GOLDEN, input_digest

pytestmark = pytest.mark.gpu

CASES = [
    ((96, 80, 64), 300, 100, 5, {}),
    ((128, 128, 128), 200, 150, 6, dict(aspect=(1.0, 4.0, 8.0), ori_mode=1, ncomp=3, scatter_deg=10.0, rho_mode=1,
                                        site_mode=1, gb_fraction=0.8)),
    ((70, 50, 90), 40, 500, 7, dict(aspect=(2.0, 1.0, 0.5), nucleation_rate=1000.0)),
]


def same(a: sg.Domain, b: sg.Domain) -> bool:
    return all(np.array_equal(np.asarray(getattr(a, f)), np.asarray(getattr(b, f)))
               for f in ("grid", "defg_quat", "defg_rho0", "rxg_quat", "rxg_site", "rxg_tincub"))


@pytest.mark.parametrize("shape,ng,nn,seed,kw", CASES)
def test_gpu_voronoi_equals_host(gpu, shape, ng, nn, seed, kw):
    host = sg.generate_domain(*shape, ng, nn, seed=seed, **kw)
    dev = sg.generate_domain(*shape, ng, nn, seed=seed, device=0, **kw)
    assert same(host, dev)
    assert len(np.unique(dev.grid)) > 0.9 * ng


@pytest.mark.slow
def test_gpu_voronoi_headline_domain(gpu):
    z = np.load(GOLDEN / "config1_512.npz")
    n, ng, nn, seed = (int(v) for v in z["gen"])
    d = sg.generate_domain(n, n, n, ng, nn, seed=seed, device=0)
    assert input_digest(d) == str(z["input_sha256"])
