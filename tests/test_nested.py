"""The nested sampler on analytic likelihoods (CPU): evidence and moments
against closed forms, determinism, and the batched proposal pool."""
import math

import numpy as np
import pytest

import lensed_gb300 as lg


def gaussian(mu, sigma):
    def f(x):
        return -0.5 * np.sum(((x - mu) / sigma) ** 2, axis=1)
    return f


@pytest.mark.parametrize("d", [2, 5])
def test_gaussian_evidence_and_moments(native, d):
    sigma = 0.05
    mu = np.full(d, 0.45)
    r = lg.nested_sample(gaussian(mu, sigma), d, nlive=300, batch=256, seed=3, tol=0.05)
    # integral of exp(-|x-mu|^2 / 2 sigma^2) over the cube (the Gaussian lies inside)
    exact = 0.5 * d * math.log(2 * math.pi * sigma ** 2)
    assert abs(r["logz"] - exact) < 4 * r["logz_err"] + 0.05, (r["logz"], exact, r["logz_err"])
    assert np.allclose(r["mean"], mu, atol=0.01)
    assert np.allclose(r["std"], sigma, rtol=0.15)
    w = np.exp(r["logwt"])
    assert abs(w.sum() - 1) < 1e-9


def test_deterministic_with_seed(native):
    f = gaussian(np.full(3, 0.6), 0.1)
    a = lg.nested_sample(f, 3, nlive=100, batch=64, seed=7)
    b = lg.nested_sample(f, 3, nlive=100, batch=64, seed=7)
    assert a["logz"] == b["logz"] and a["ncall"] == b["ncall"]


def test_invalid_options(native):
    with pytest.raises(lg.LensedError):
        lg.nested_sample(gaussian(np.full(4, 0.5), 0.1), 4, nlive=3)


def test_callback_errors_propagate(native):
    def bad(x):
        raise RuntimeError("boom")
    with pytest.raises(RuntimeError):
        lg.nested_sample(bad, 2, nlive=20, batch=8)
