"""Host-side logic of the C ABI: weights, priors and the parameter map."""
import math

import numpy as np
import pytest

import lensed_gb300 as lg
from oracle import oracle


def test_make_weight_matches_oracle(native):
    rng = np.random.Generator(np.random.PCG64(0))
    img = rng.uniform(1, 100, size=(20, 30)).astype(np.float32)
    gain = rng.uniform(0.5, 2, size=img.shape).astype(np.float32)
    xw = rng.uniform(0.5, 1.5, size=img.shape).astype(np.float32)
    mask = (rng.random(img.shape) < 0.1).astype(np.int32)
    for kw in ({"gain_value": 1.7, "offset": 2.9633}, {"gain": gain, "offset": 0.5, "xweight": xw, "mask": mask},
               {"weight_map": gain, "mask": mask}):
        w, masked = lg.make_weight(img, **kw)
        want = oracle.make_weight(img, **kw)
        assert np.array_equal(w, want)
        assert masked == int((want == 0).sum())


def test_norm_prior_quantile_restates_reference():
    # Abramowitz & Stegun 26.2.23 as in src/prior/norm.c:9-16; |error| < 4.5e-4
    from statistics import NormalDist

    nd = NormalDist()
    for u in (0.001, 0.1, 0.3, 0.5 - 1e-9, 0.7, 0.95, 0.999):
        t = math.sqrt(-2 * math.log(u if u < 0.5 else 1 - u))
        t = t - ((0.010328 * t + 0.802853) * t + 2.515517) / (((0.001308 * t + 0.189269) * t + 1.432788) * t + 1.)
        v = -t if u < 0.5 else t
        assert abs(v - nd.inv_cdf(u)) < 4.5e-4
