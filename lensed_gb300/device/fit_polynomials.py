"""Derive the polynomial coefficients of the paired-ray atan and atanh in
lg_prelude.cuh (run by hand; prints the float32 coefficients as C hex
literals and the accuracy of their FP32 Horner evaluation).

* atan(r) = r P(r^2) on r in [0, 1], P of degree 9;
* atanh(v) = v Q(v^2) on v in [0, 1/2], Q of degree 6.

Method: least squares on Chebyshev-distributed points for the relative
error of the function, reweighted a few dozen times towards equal ripple
(a Lawson-style iteration approximating the minimax fit), with the
constant term then pinned to 1.  Only numpy is needed.

Usage: python lensed_gb300/device/fit_polynomials.py
"""
import numpy as np


def fit_relative(f, a, b, deg, n=20000, iters=30):
    s = 0.5 * (a + b) + 0.5 * (b - a) * np.cos(np.linspace(0, np.pi, n))
    g = 1.0 / f(s)
    w = np.ones_like(s)
    for _ in range(iters):
        V = np.vander(s, deg + 1, increasing=True)
        c, *_ = np.linalg.lstsq(V * (w * g)[:, None], f(s) * w * g, rcond=None)
        e = (V @ c - f(s)) * g
        w = w * (np.abs(e) / np.abs(e).max() + 1e-3) ** 0.5
        w /= w.max()
    return c, np.abs(e).max()


def horner32(c, s):
    """Horner in FP32 with one rounding per step (an fma)."""
    c32 = c.astype(np.float32)
    r = np.full_like(s, c32[-1])
    for k in range(len(c32) - 2, -1, -1):
        r = (r.astype(np.float64) * s + c32[k]).astype(np.float32)
    return r


def report(name, f, ref, a, b, deg):
    c, e = fit_relative(f, a, b, deg)
    c[0] = 1.0
    x = np.linspace(0, np.sqrt(b), 200001).astype(np.float32)
    y = (x * horner32(c, (x * x).astype(np.float32))).astype(np.float32)
    want = ref(x.astype(np.float64))
    rel = (np.abs(y - want)[1:] / np.abs(want[1:])).max()
    print(f"{name}: degree {deg}, fit error {e:.3g}, FP32 max relative error {rel:.3g}")
    print("  coefficients (s^0 first):", ", ".join(float.hex(float(np.float32(v))) for v in c))


def main():
    atan_q = lambda s: np.where(s > 0, np.arctan(np.sqrt(s)) / np.sqrt(np.maximum(s, 1e-300)), 1.0)
    atanh_q = lambda s: np.where(s > 0, np.arctanh(np.sqrt(s)) / np.sqrt(np.maximum(s, 1e-300)), 1.0)
    report("atan", atan_q, np.arctan, 0.0, 1.0, 9)
    report("atanh", atanh_q, np.arctanh, 0.0, 0.25, 6)


if __name__ == "__main__":
    main()
