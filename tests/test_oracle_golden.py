"""Pin the CPU oracle against the reference's own test images.

tests/golden/fixtures.npz holds the 16 noiseless model images of the
reference's batch tests (tests/{lens,source,foreground}/*.ini, 100x100) with
their parameters.  The FP32 and FP64 oracles must reproduce them; the
tolerances are the measured agreement of a rule-g3k7 render with images made
by an older Lensed release (max relative error over pixels above 1e-6 of the
peak: <= 3.2e-5 for lenses, <= 1.2e-4 for the far tails of the sources).
"""
import numpy as np
import pytest

from lensed_gb300 import quadrature
from oracle.oracle import Oracle

TOL = {"lens": 5e-5, "foreground": 5e-6, "source": 2e-4}


def cases(golden):
    return [str(c) for c in golden["cases"]]


@pytest.mark.parametrize("precision", [32, 64])
def test_oracle_reproduces_reference_images(golden, precision):
    rule = quadrature.rule("g3k7")
    for case in cases(golden):
        plugins = [str(p) for p in golden[f"{case}__plugins"]]
        params = golden[f"{case}__params"]
        ref = golden[f"{case}__image"].astype(np.float64)
        o = Oracle(plugins, 100, 100, rule, precision=precision)
        v, _, _ = o.render(params)
        big = np.abs(ref) > 1e-6 * np.abs(ref).max()
        rel = (np.abs(v - ref)[big] / np.abs(ref[big])).max()
        assert rel <= TOL[case.split("__")[0]], (case, rel)
        assert abs(v.sum() - ref.sum()) <= 1e-5 * abs(ref.sum()), case


def test_epl_isothermal_equals_sie():
    """Known answer from the reference's fixtures: the EPL with t = 1 is the SIE."""
    rule = quadrature.rule("g3k7")
    src = [50.5, 50.5, 5.0, -5.0, 1.0, 1.0, 0.0]
    a = Oracle(["sie", "sersic"], 100, 100, rule, precision=64).render([50.5, 50.5, 20.0, 0.8, 45.0] + src)[0]
    b = Oracle(["epl", "sersic"], 100, 100, rule, precision=64).render([50.5, 50.5, 20.0, 1.0, 0.8, 45.0] + src)[0]
    assert np.abs(a - b).max() <= 1e-6 * np.abs(a).max()
    a = Oracle(["sie_plus_shear", "sersic"], 100, 100, rule, precision=64).render(
        [50.5, 50.5, 20.0, 0.8, 45.0, 0.1, -0.1] + src)[0]
    b = Oracle(["epl_plus_shear", "sersic"], 100, 100, rule, precision=64).render(
        [50.5, 50.5, 20.0, 1.0, 0.8, 45.0, 0.1, -0.1] + src)[0]
    assert np.abs(a - b).max() <= 1e-6 * np.abs(a).max()


def test_fp32_oracle_close_to_fp64(golden):
    rule = quadrature.rule("g3k7")
    for case in cases(golden):
        plugins = [str(p) for p in golden[f"{case}__plugins"]]
        params = golden[f"{case}__params"]
        a = Oracle(plugins, 100, 100, rule, precision=32).render(params)[0]
        b = Oracle(plugins, 100, 100, rule, precision=64).render(params)[0]
        big = np.abs(b) > 1e-6 * np.abs(b).max()
        assert (np.abs(a - b)[big] / np.abs(b[big])).max() < 2e-4, case


def test_blank_loglike_is_minus_half_chi2():
    """logL = -chi^2/2 with no normalisation term (src/nested.c:115)."""
    rule = quadrature.rule("point")
    img = np.zeros((10, 10), np.float32)
    w = np.full((10, 10), 2.0, np.float32)
    o = Oracle(["sky"], 10, 10, rule, image=img, weight=w, precision=64)
    ll = o.loglike([[3.0, 0.0, 0.0]])[0]
    assert ll == pytest.approx(-0.5 * 100 * 2.0 * 9.0)
