"""The restatement (oracle) against the reference's own code compiled on the
host (oracle/_ref, built from the reference sources by oracle/build_ref.py).

With the same elementary functions (math="cr"), the reference's kernels and
generated compute()/set_params and the oracle must produce bit-identical
images and logL equal to the last bits of the FP64 sum.  Skipped when the
reference-built libraries are absent.
"""
import numpy as np
import pytest

from lensed_gb300 import quadrature, workloads
from oracle import ref as R
from oracle.oracle import Oracle

pytestmark = pytest.mark.skipif(not R.available(), reason="reference-built checker not present")


def test_reference_images_restated_bitwise(golden):
    rule = quadrature.rule("g3k7")
    n = 0
    for case in [str(c) for c in golden["cases"]]:
        plugins = [("sersic" if p == "sersic_old" else str(p)) for p in golden[f"{case}__plugins"]]
        params = golden[f"{case}__params"]
        ref = R.Reference(plugins, 100, 100, rule, threads=4)
        a = ref.render(params)
        b = Oracle(plugins, 100, 100, rule, precision=32, threads=4).render(params)
        assert np.array_equal(a[0], b[0].astype(np.float32)), case
        assert np.array_equal(a[1], b[1].astype(np.float32)), case
        n += 1
    assert n == 16


@pytest.mark.parametrize("name", ["small", "config2"])
def test_workload_loglike_restated(name):
    s = getattr(workloads, name)()
    cand = workloads.draw_candidates(s, 3, seed=2)
    ref = R.Reference.for_system(s, threads=8, math="cr")
    o = Oracle(s.plugins, s.width, s.height, quadrature.rule(s.rule), psf=s.psf, image=s.image, weight=s.weight,
               precision=32, threads=8)
    a, b = ref.loglike(cand), o.loglike(cand)
    assert np.abs(a - b).max() <= 1e-9 * np.abs(b).max()
    va, _, ca = ref.render(cand[0])
    vb, _, cb = o.render(cand[0])
    assert np.array_equal(va, vb.astype(np.float32))
    if ca is not None:
        assert np.array_equal(ca, cb.astype(np.float32))


def test_image_plane_prior_and_even_psf_restated():
    rule = quadrature.rule("sub3")
    params = [24.3, 23.8, 9.0, 0.75, 40.0, 14.0, 30.0, 2.0, -1.0, 2.0, 0.8, 30.0]
    a = R.Reference([("sie", 0), ("sersic", 1)], 48, 48, rule).render(params)[0]
    b = Oracle([("sie", 0), ("sersic", 1)], 48, 48, rule, precision=32).render(params)[0]
    assert np.array_equal(a, b.astype(np.float32))
    psf = workloads.psf_gauss_wings(8, 2.0)[:, :7].copy()
    rule = quadrature.rule("sub2")
    p = [20.3, 18.7, 8.0, 0.7, 35.0, 0.05, -0.03, 21.0, 18.0, 3.0, -2.0, 0.8, 20.0]
    ra = R.Reference(["sie_plus_shear", "gauss"], 45, 52, rule, psf=psf).render(p)
    ob = Oracle(["sie_plus_shear", "gauss"], 45, 52, rule, psf=psf, precision=32).render(p)
    assert np.array_equal(ra[0], ob[0].astype(np.float32))
    assert np.array_equal(ra[2], ob[2].astype(np.float32))
