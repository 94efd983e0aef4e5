"""Accuracy of the paired-ray exp, log, square root and reciprocal of the
fast evaluation modules (SFU ex2/lg2 with a first-order correction; SFU
sqrt and rcp) against double precision.

Bounds, for results in the normal float range:
* exp: relative error <= 4 ulp (2^-21), the class of CUDA's expf (2 ulp)
  plus the SFU's own approximation error;
* log: absolute error <= 3e-7 or relative error <= 4 ulp, whichever is
  larger (the correction leaves an absolute error of about 2^-22);
* sqrt and 1/x: relative error <= 2^-22 (x normal; 1/x for |x| <= 2^126);
* atan: relative error <= 2^-22; atanh: relative error <= 2^-22 for
  |v| <= 1/2 and absolute error <= 3e-7 above (the deflection angles of
  the SIE family, added to pixel positions whose own rounding is ~1e-5);
* special values: exp(-inf) = 0, exp(+inf) = exp(overflowing x) = inf,
  exp(NaN) = NaN, results below 2^-126 flushed to 0; log(0) = -inf,
  log(inf) = inf, log(negative) = NaN, log of huge finite x still accurate.
"""
import ctypes as C

import numpy as np
import pytest

import lensed_gb300 as lg

pytestmark = pytest.mark.gpu


def run(fn, x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty_like(x)
    fp = C.POINTER(C.c_float)
    rc = lg.lib().lg_probe_pair_math(0, fn, x.ctypes.data_as(fp), x.size, out.ctypes.data_as(fp))
    assert rc == 0, lg.lib().lg_last_error(None)
    return out


def test_exp_accuracy(native):
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(-87, 88.5, 400000), rng.uniform(-1, 1, 100000),
                        np.linspace(-87.3, 88.7, 20001)]).astype(np.float32)
    got = run(0, x).astype(np.float64)
    want = np.exp(x.astype(np.float64))
    normal = (want >= 2.0**-126) & (want < 3.4e38)
    rel = np.abs(got[normal] - want[normal]) / want[normal]
    print(f"exp: max rel error {rel.max():.3g} = {rel.max() / 2**-24:.2f} ulp(half) units")
    assert rel.max() <= 2.0**-21


def test_log_accuracy(native):
    rng = np.random.default_rng(2)
    x = np.concatenate([np.exp(rng.uniform(-87, 88.7, 400000)), rng.uniform(0.5, 2, 100000),
                        [1.0, 2.0, 0.5, 1e-37, 3e38, 1 + 2**-23, 1 - 2**-24]]).astype(np.float32)
    got = run(1, x).astype(np.float64)
    want = np.log(x.astype(np.float64))
    err = np.abs(got - want)
    ok = (err <= 3e-7) | (err <= 2.0**-21 * np.abs(want))
    i = np.argmax(err)
    print(f"log: max abs error {err.max():.3g} at x={x[i]:.6g}")
    assert ok.all(), x[~ok][:10]


def test_special_values(native):
    e = run(0, [-np.inf, np.inf, np.nan, 100.0, -100.0, 0.0, -0.0, 89.0, -88.0])
    assert e[0] == 0 and np.isposinf(e[1]) and np.isnan(e[2]) and np.isposinf(e[3]) and e[4] == 0
    assert e[5] == 1 and e[6] == 1 and np.isposinf(e[7]) and 0 <= e[8] < 2.0**-126
    lo = run(1, [0.0, np.inf, -1.0, np.nan, 3.4e38, 2e-38])
    assert np.isneginf(lo[0]) and np.isposinf(lo[1]) and np.isnan(lo[2]) and np.isnan(lo[3])
    assert abs(lo[4] - np.log(3.4e38)) < 1e-5 * np.log(3.4e38)
    assert abs(lo[5] - np.log(2e-38)) < 1e-5 * abs(np.log(2e-38))


def test_sqrt_and_reciprocal(native):
    rng = np.random.default_rng(3)
    x = np.concatenate([np.exp(rng.uniform(-87, 87, 300000)), rng.uniform(0.25, 4, 100000)]).astype(np.float32)
    for fn, ref in ((2, np.sqrt), (3, lambda v: 1.0 / v)):
        got = run(fn, x).astype(np.float64)
        want = ref(x.astype(np.float64))
        rel = np.abs(got - want) / want
        print(f"fn {fn}: max rel error {rel.max():.3g}")
        assert rel.max() <= 2.0**-22
    s = run(2, [0.0, np.inf, -1.0, np.nan])
    assert s[0] == 0 and np.isposinf(s[1]) and np.isnan(s[2]) and np.isnan(s[3])
    r = run(3, [0.0, np.inf, -2.0])
    assert np.isposinf(r[0]) and r[1] == 0 and r[2] == -0.5


def test_atan_and_atanh(native):
    rng = np.random.default_rng(4)
    z = np.concatenate([rng.uniform(-1, 1, 200000), np.exp(rng.uniform(-20, 20, 200000)) * rng.choice([-1, 1], 200000),
                        [0.0, -0.0, 1.0, -1.0, 1e-30, 1e30]]).astype(np.float32)
    got = run(4, z).astype(np.float64)
    want = np.arctan(z.astype(np.float64))
    nz = want != 0
    rel = np.abs(got[nz] - want[nz]) / np.abs(want[nz])
    print(f"atan: max rel error {rel.max():.3g}")
    assert rel.max() <= 2.0**-22 and np.all(got[~nz] == 0)
    v = np.concatenate([rng.uniform(-0.999, 0.999, 300000), rng.uniform(-1e-3, 1e-3, 50000),
                        [0.0, 0.5, -0.5, 0.50001, 0.9999999]]).astype(np.float32)
    got = run(5, v).astype(np.float64)
    want = np.arctanh(v.astype(np.float64))
    small = np.abs(v) <= 0.5
    nz = small & (want != 0)
    rel = np.abs(got[nz] - want[nz]) / np.abs(want[nz])
    absd = np.abs(got[~small] - want[~small])
    print(f"atanh: max rel error {rel.max():.3g} (|v| <= 1/2), max abs error {absd.max():.3g} above")
    assert rel.max() <= 2.0**-22 and absd.max() <= 3e-7
    sp = run(5, [1.0, -1.0, 1.5, np.nan])
    assert np.isposinf(sp[0]) and np.isneginf(sp[1]) and np.isnan(sp[2]) and np.isnan(sp[3])
    sa = run(4, [np.inf, -np.inf, np.nan])
    assert abs(sa[0] - np.pi / 2) < 1e-7 and abs(sa[1] + np.pi / 2) < 1e-7 and np.isnan(sa[2])
