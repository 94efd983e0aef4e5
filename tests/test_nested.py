"""The nested sampler on analytic likelihoods (CPU): evidence and moments
against closed forms, determinism, and the batched proposal pool."""
import math
import os

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


def test_zero_likelihood_outside_a_box(native):
    """logL = -inf on 90% of the prior (a box cut, as bound rejection of
    the priors gives): such draws are dropped from the initial live points
    and counted out of the starting prior volume; the evidence is that of
    the Gaussian inside the box (40 seeds: -6.591 +- 0.027 against
    -6.612)."""
    d, sigma = 3, 0.05
    mu = np.array([0.3, 0.5, 0.6])
    lo, hi = np.array([0.0, 0.0, 0.0]), np.array([1.0, 1.0, 0.1])  # the box: 10% of the cube

    def f(x):
        inside = np.all((x >= lo + np.array([0, 0, 0.55])) & (x <= hi + np.array([0, 0, 0.55])), axis=1)
        ll = -0.5 * np.sum(((x - mu) / sigma) ** 2, axis=1)
        return np.where(inside, ll, -np.inf)

    r = lg.nested_sample(f, d, nlive=200, batch=128, seed=4, tol=0.05)
    # the box (z in [0.55, 0.65]) holds the Gaussian's z-marginal within +-1 sigma
    from math import erf, sqrt
    mass = 0.5 * (erf(0.05 / (sigma * sqrt(2))) - erf(-0.05 / (sigma * sqrt(2))))
    exact = 0.5 * d * math.log(2 * math.pi * sigma ** 2) + math.log(mass)
    assert abs(r["logz"] - exact) < 4 * r["logz_err"] + 0.05, (r["logz"], exact, r["logz_err"])
    b = lg.nested_sample(f, d, nlive=200, batch=128, seed=4, tol=0.05)
    assert b["logz"] == r["logz"] and b["ncall"] == r["ncall"]


def test_invalid_options(native):
    with pytest.raises(lg.LensedError):
        lg.nested_sample(gaussian(np.full(4, 0.5), 0.1), 4, nlive=3)


def test_callback_errors_propagate(native):
    def bad(x):
        raise RuntimeError("boom")
    with pytest.raises(RuntimeError):
        lg.nested_sample(bad, 2, nlive=20, batch=8)


def test_wrapped_dimension(native):
    """A periodic parameter (the prior keyword "wrap"): the likelihood in
    dimension 0 is a Gaussian centred on the boundary 0 = 1 of a periodic
    coordinate; with wrap on, proposals leaving the cube there re-enter on
    the other side, and the evidence is the full Gaussian integral."""
    sigma = 0.05

    def f(x):
        d0 = x[:, 0] - np.round(x[:, 0])  # periodic distance to 0 = 1
        return -0.5 * (d0 / sigma) ** 2 - 0.5 * np.sum(((x[:, 1:] - 0.5) / sigma) ** 2, axis=1)

    exact = 1.5 * math.log(2 * math.pi * sigma ** 2)
    r = lg.nested_sample(f, 3, nlive=300, batch=256, seed=11, tol=0.05, wrap=[1, 0, 0])
    assert abs(r["logz"] - exact) < 4 * r["logz_err"] + 0.05, (r["logz"], exact)
    w = np.exp(r["logwt"])
    x0 = r["samples"][:, 0]
    # posterior mass on both sides of the boundary, none in the middle
    assert w[x0 < 0.2].sum() > 0.3 and w[x0 > 0.8].sum() > 0.3
    assert w[(x0 > 0.3) & (x0 < 0.7)].sum() < 1e-3


def test_checkpoint_and_resume_continue_exactly(native, tmp_path):
    """A run stopped after 400 iterations (checkpoints every 150) and resumed
    from its state file ends with the same evidence, calls and samples as the
    uninterrupted run: the state holds the live and dead points, the
    evidence accumulators, the RNG and the pool of evaluated proposals."""
    f = gaussian(np.array([0.3, 0.6, 0.45]), 0.07)
    common = dict(nlive=200, batch=64, seed=5, tol=0.05)
    full = lg.nested_sample(f, 3, **common)
    path = str(tmp_path / "state.bin")
    part = lg.nested_sample(f, 3, maxiter=400, checkpoint=path, checkpoint_every=150, **common)
    assert part["niter"] == 400 and os.path.exists(path)
    rest = lg.nested_sample(f, 3, checkpoint=path, resume=1, **common)
    assert rest["logz"] == full["logz"] and rest["ncall"] == full["ncall"] and rest["niter"] == full["niter"]
    assert np.array_equal(rest["samples"], full["samples"])
    # a finished state resumes to the same result at once
    again = lg.nested_sample(f, 3, checkpoint=path, resume=1, **common)
    assert again["logz"] == full["logz"] and again["ncall"] == full["ncall"]
    # a state for another problem size, or a file of another format, is an
    # error rather than a silent fresh start
    with pytest.raises(lg.LensedError, match="another dimension"):
        lg.nested_sample(gaussian(np.full(2, 0.5), 0.1), 2, checkpoint=path, resume=1, nlive=100, batch=64, seed=5)
    with open(path, "r+b") as fh:
        fh.seek(7)
        fh.write(b"3")  # the previous format version
    with pytest.raises(lg.LensedError, match="format version"):
        lg.nested_sample(f, 3, checkpoint=path, resume=1, **common)
    # no file at all: a fresh run
    fresh = lg.nested_sample(f, 3, checkpoint=str(tmp_path / "none.bin"), resume=1, **common)
    assert fresh["logz"] == full["logz"]


def test_plateaus_of_a_stepped_likelihood(native, tmp_path):
    """A likelihood in steps of 0.5 (ties everywhere, a plateau at the top):
    tied lowest points shrink the volume by 1 / (nlive - j), the run stops
    when every live point sits on the top plateau, and the evidence matches
    the closed form (20 seeds: -4.153 +- 0.025 against -4.133); a resumed
    run continues through a plateau exactly."""
    sigma, mu = 0.05, np.array([0.5, 0.45])

    def f(x):
        return np.round(-np.sum(((x - mu) / sigma) ** 2, axis=1)) / 2

    # round(r^2 / sigma^2) = k on a ring of area pi sigma^2 (half that for k = 0)
    exact = math.log(math.pi * sigma ** 2 * (0.5 + sum(math.exp(-k / 2) for k in range(1, 2000))))
    common = dict(nlive=200, batch=128, seed=3, tol=0.01)
    full = lg.nested_sample(f, 2, **common)
    assert abs(full["logz"] - exact) < 4 * full["logz_err"], (full["logz"], exact, full["logz_err"])
    path = str(tmp_path / "state.bin")
    part = lg.nested_sample(f, 2, maxiter=700, checkpoint=path, **common)
    assert part["niter"] == 700
    rest = lg.nested_sample(f, 2, checkpoint=path, resume=1, **common)
    assert rest["logz"] == full["logz"] and rest["ncall"] == full["ncall"] and rest["niter"] == full["niter"]


def test_constant_efficiency_mode(native, tmp_path):
    """ceff = 1 (the reference's ceff option): the bound's volume follows
    the target acceptance efr -- about 1 / efr likelihood calls per
    replacement -- and a resumed run continues exactly (the enlargement is
    in the state)."""
    d, sigma = 5, 0.05
    f = gaussian(np.full(d, 0.45), sigma)
    exact = 0.5 * d * math.log(2 * math.pi * sigma ** 2)
    common = dict(nlive=300, batch=256, seed=2, tol=0.05, ceff=1, efr=0.3)
    r = lg.nested_sample(f, d, **common)
    assert 2.5 < r["ncall"] / r["niter"] < 4.5, r["ncall"] / r["niter"]
    assert abs(r["logz"] - exact) < 4 * r["logz_err"] + 0.1, (r["logz"], exact)
    path = str(tmp_path / "state.bin")
    lg.nested_sample(f, d, maxiter=1500, checkpoint=path, **common)
    rest = lg.nested_sample(f, d, checkpoint=path, resume=1, **common)
    assert rest["logz"] == r["logz"] and rest["ncall"] == r["ncall"]


def test_multi_ellipsoid_bound_on_two_modes(native):
    """Two well separated modes (d = 4): the multi-ellipsoidal bound (MultiNest's
    multi-modal mode) finds the evidence with far fewer likelihood calls than
    one ellipsoid spanning both modes and the empty space between them."""
    d, sigma = 4, 0.03

    def f(x):
        a = -0.5 * np.sum(((x - 0.3) / sigma) ** 2, axis=1)
        b = -0.5 * np.sum(((x - 0.7) / sigma) ** 2, axis=1)
        return np.logaddexp(a, b) + math.log(0.5)

    exact = 0.5 * d * math.log(2 * math.pi * sigma ** 2)
    common = dict(nlive=400, batch=256, seed=2, tol=0.1)
    one = lg.nested_sample(f, d, **common)
    many = lg.nested_sample(f, d, max_ellipsoids=8, **common)
    print(f"two modes d={d}: exact {exact:.3f}; one ellipsoid {one['logz']:.3f}+-{one['logz_err']:.3f} "
          f"({one['ncall']} calls); up to 8 {many['logz']:.3f}+-{many['logz_err']:.3f} ({many['ncall']} calls)")
    for r in (one, many):
        assert abs(r["logz"] - exact) < 4 * r["logz_err"] + 0.1
    assert many["ncall"] < 0.5 * one["ncall"]
    # both modes carry about half of the posterior
    w = np.exp(many["logwt"])
    assert 0.35 < w[many["samples"][:, 0] < 0.5].sum() < 0.65


def test_multi_ellipsoid_resume_is_exact(native, tmp_path):
    f = gaussian(np.array([0.3, 0.6, 0.45]), 0.07)
    common = dict(nlive=200, batch=64, seed=5, tol=0.05, max_ellipsoids=4)
    full = lg.nested_sample(f, 3, **common)
    path = str(tmp_path / "state.bin")
    lg.nested_sample(f, 3, maxiter=333, checkpoint=path, **common)
    rest = lg.nested_sample(f, 3, checkpoint=path, resume=1, **common)
    assert rest["logz"] == full["logz"] and rest["ncall"] == full["ncall"]
