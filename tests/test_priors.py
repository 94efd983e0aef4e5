"""Parameter space and priors on the CPU: the product's plugin tables
against the reference's (tests/golden/plugin_params.json, generated from
objects/*.cl by make_plugin_params.py), and the oracle's restatement of the
prior transform (src/prior/*.c, src/nested.c:42-61)."""
import json
import math
import os

import numpy as np
import pytest

import lensed_gb300 as lg
from oracle.priors import ParamSpace, apply, norm_quantile, parse_prior

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = json.load(open(os.path.join(HERE, "golden", "plugin_params.json")))
KINDS = {"LENS": 0, "SOURCE": 1, "FOREGROUND": 2}


@pytest.mark.parametrize("plugin", sorted(TABLE))
def test_plugin_tables_match_reference(native, plugin):
    got = lg.plugin_params(plugin)
    want = TABLE[plugin]["params"]
    assert [g[0] for g in got] == [w[0] for w in want]
    for (n, t, lo, hi, dv), (wn, wt, wlo, whi, wdv) in zip(got, want):
        assert t == wt, (plugin, n)
        assert (np.float32(lo), np.float32(hi)) == (np.float32(wlo), np.float32(whi)), (plugin, n)
        assert np.float32(dv) == np.float32(wdv) and math.copysign(1, dv) == math.copysign(1, wdv), (plugin, n)


def test_norm_quantile_is_the_published_approximation():
    scipy_stats = pytest.importorskip("scipy.stats")
    u = np.concatenate([np.linspace(1e-6, 1 - 1e-6, 2001), [1e-300, 1e-12, 0.5, 1 - 1e-12]])
    q = np.array([norm_quantile(x) for x in u])
    # Abramowitz & Stegun 26.2.23: absolute error below 4.5e-4
    assert np.abs(q - scipy_stats.norm.ppf(u)).max() < 4.5e-4
    # antisymmetric about u = 1/2 up to the rounding of 1 - u (relative 1e-16 / u)
    mid = (u > 1e-3) & (u < 1 - 1e-3) & (u != 0.5)  # at 0.5 both take the upper branch
    back = np.array([norm_quantile(1 - x) for x in u[mid]])
    assert np.abs(q[mid] + back).max() < 1e-13


def test_prior_parse_and_apply():
    assert apply(parse_prior("unif 2 6"), 0.25) == 3.0
    assert apply(parse_prior("3.5"), 0.9) == 3.5
    p = parse_prior("wrap norm 1 2")
    assert p.wrap and p.kind == "norm" and (p.lower(), p.upper()) == (-13.0, 15.0)
    # the approximation is 1e-7 off zero at u = 1/2 (its upper branch)
    assert abs(apply(p, 0.5) - 1.0) < 2 * 1.1e-7
    assert parse_prior("image unif 0 1").image
    with pytest.raises(ValueError):
        parse_prior("unif 1")


def test_param_space_map_and_bounds():
    objs = [("lens", "sie", {"x": "unif 10 20", "y": "norm 15 1", "r": "unif 5 10", "q": "norm 0.9 0.1",
                             "pa": "unif 0 180"}),
            ("sky", "sky", {"bg": "unif 0 1"})]
    ps = ParamSpace(objs, TABLE)
    ids = [ps.params[k].id for k in ps.pmap]
    # sky.dx, sky.dy default to -0 (delta priors): derived, at the end
    assert ids == ["lens.x", "lens.y", "lens.r", "lens.q", "lens.pa", "sky.bg", "sky.dx", "sky.dy"]
    assert ps.ndims == 6
    q = ps.params[3]
    assert q.bounded and (q.lower, q.upper) == (0.0, 1.0)
    r = ps.params[2]
    assert r.bounded and r.upper == math.inf
    assert not ps.params[0].bounded
    cube = np.array([[0.5, 0.5, 0.5, 0.5, 0.5, 0.5], [0.5, 0.5, 0.5, 0.999, 0.5, 0.5]])
    phys, bad = ps.transform(cube)
    assert list(bad) == [False, True]  # q = 0.9 + 0.1 * 3.09 > 1
    assert phys[0, 0] == 15.0 and abs(phys[0, 1] - 15.0) < 2e-7 and math.copysign(1, phys[0, 6]) == -1
