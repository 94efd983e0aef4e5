"""Quadrature rules: generated from mathematics, identical to the reference's."""
import os
import re

import numpy as np
import pytest

from lensed_gb300 import quadrature
from oracle.build_ref import REF as LENSED_SOURCE

# the reference tree (LENSED_SOURCE); the test is skipped where it is absent
REF = os.path.join(LENSED_SOURCE, "src", "quad")


def test_table_matches_generator():
    pytest.importorskip("mpmath")
    gen = quadrature.generate()
    for name, r in gen.items():
        assert quadrature.rule(name) == r, name


def test_rule_sizes_and_normalisation():
    sizes = {"point": 1, "sub2": 4, "sub3": 9, "sub4": 16, "sub5": 25, "gm75": 17, "g3k7": 49, "g5k11": 121,
             "g7k15": 225}
    for name, n in sizes.items():
        r = quadrature.rule(name)
        assert r.size == n
        assert sum(r.weights) == pytest.approx(1.0, abs=1e-14)
        pts = np.array(r.points)
        assert np.all(np.abs(pts) < 0.5)


def test_exactness_on_polynomials():
    # Gauss-Kronrod 2n+1 points integrate x^k exactly up to 3n+1 on [-1/2, 1/2]
    for name, deg in (("g3k7", 10), ("g5k11", 16), ("g7k15", 22)):
        r = quadrature.rule(name)
        x = np.array(r.points)[:, 0]
        w = np.array(r.weights)
        for k in range(0, deg + 1, 2):
            exact = 2 * 0.5 ** (k + 1) / (k + 1)
            assert np.dot(w, x ** k) == pytest.approx(exact, rel=1e-12), (name, k)
        # the error weights annihilate polynomials the Gauss rule integrates
        e = np.array(r.errors)
        assert abs(np.dot(e, np.ones_like(x))) < 1e-14


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference sources not present")
def test_same_numbers_as_reference_tables():
    for name in ["point", "sub2", "sub4", "gm75", "g3k7", "g5k11", "g7k15"]:
        t = open(os.path.join(REF, f"{name}.c")).read()

        def arr(suf):
            m = re.search(r"QUAD_\w+_" + suf + r"\[\](?:\[2\])?\s*=\s*\{(.*?)\};", t, re.S)
            return [float(v) for v in re.findall(r"[-+]?\d+\.?\d*(?:[eE][-+]?\d+)?", m.group(1))]

        r = quadrature.rule(name)
        assert np.array_equal(np.array(arr("PTS")), np.array(r.points).ravel()), name
        assert np.array_equal(np.array(arr("WHT")), np.array(r.weights)), name
        assert np.array_equal(np.array(arr("ERR")), np.array(r.errors)), name
