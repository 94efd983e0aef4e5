"""The unit-cube prior transform on the GPU (src/nested.c:42-61) against the
oracle's restatement (oracle/priors.py), through the host and device entry
points and the reference-signature loglike() callback.

* uniform and delta priors are exact IEEE double arithmetic: bit-exact;
* normal priors go through a double log; CUDA's and the host's may differ
  in the last bit, so values agree within 1e-14 relative to sigma;
* a value outside the parameter bounds is rejected (logL = -inf; the host
  API returns NaN parameters), where the reference would redraw forever;
* accepted points have exactly the logL of lg_eval_batch on the same
  physical values.
"""
import json
import os

import numpy as np
import pytest

import lensed_gb300 as lg
from oracle.priors import ParamSpace

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = json.load(open(os.path.join(HERE, "golden", "plugin_params.json")))

OBJECTS = [
    ("lens", "sie", {"x": "unif 20 28", "y": "norm 24 1.5", "r": "unif 5 12", "q": "norm 0.9 0.1",
                     "pa": "wrap unif 0 180"}),
    ("src", "sersic", {"x": "norm 24 3", "y": "unif 18 30", "r": "unif 1 4", "mag": "-2.5", "n": "norm 2 2",
                       "q": "unif 0.4 1", "pa": "unif 0 180"}),
    ("sky", "sky", {"bg": "norm 5 0.5"}),
]


def _ctx(max_batch=64, flags=0):
    W = H = 48
    rng = np.random.default_rng(2)
    image = rng.normal(5.0, 1.0, size=(H, W)).astype(np.float32)
    weight = np.ones((H, W), np.float32)
    return lg.Context(image, weight, OBJECTS, rule="sub3", max_batch=max_batch, flags=flags)


def _cube(nd, B=200, seed=11):
    rng = np.random.default_rng(seed)
    cube = rng.random((B, nd))
    cube[0] = 0.5
    cube[1] = 1e-300
    cube[2] = 1 - 2**-53
    cube[3, :] = 0.999  # q = 0.9 + 0.1 * 3.09 > 1: rejected
    return cube


def _check_phys(ps, got, want):
    kinds = [ps.params[k].prior.kind for k in ps.pmap]
    sig = np.array([ps.params[k].prior.b if ps.params[k].prior.kind == "norm" else 0.0 for k in ps.pmap])
    for i, kind in enumerate(kinds):
        g, w = got[:, i], want[:, i]
        if kind == "norm":
            assert np.all(np.abs(g - w) <= 1e-14 * (np.abs(w) + sig[i])), ps.params[ps.pmap[i]].id
        else:
            assert np.array_equal(g.view(np.int64), w.view(np.int64)), ps.params[ps.pmap[i]].id


@pytest.mark.parametrize("flags", [0, lg.LG_FLAG_NO_GRAPH])
def test_cube_transform_matches_oracle(native, flags):
    ctx = _ctx(flags=flags)
    ps = ParamSpace(OBJECTS, TABLE)
    assert ctx.ids == [ps.params[k].id for k in ps.pmap] and ctx.ndims == ps.ndims
    cube = _cube(ctx.ndims)
    want, bad = ps.transform(cube)
    ll, phys = ctx.eval_cube(cube)  # 200 points in chunks of max_batch = 64
    assert bad[3] and bad.sum() >= 1
    assert np.array_equal(np.isneginf(ll), bad)
    assert np.all(np.isnan(phys[bad]))
    _check_phys(ps, phys[~bad], want[~bad])
    assert np.array_equal(ll[~bad], np.concatenate([ctx.eval_batch(p) for p in np.array_split(phys[~bad], 4)]))
    ctx.close()


def test_cube_device_entry_point(native):
    torch = pytest.importorskip("torch")
    ctx = _ctx()
    ps = ParamSpace(OBJECTS, TABLE)
    cube = _cube(ctx.ndims, B=64, seed=12)
    d_cube = torch.tensor(cube, dtype=torch.float64, device="cuda")
    d_phys = torch.empty((64, ctx.npars), dtype=torch.float64, device="cuda")
    d_logL = torch.empty(64, dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())  # the inputs were written on the current stream
    ctx.eval_cube_device(d_cube.data_ptr(), 64, d_phys.data_ptr(), d_logL.data_ptr(), s.cuda_stream)
    s.synchronize()
    ll, phys = d_logL.cpu().numpy(), d_phys.cpu().numpy()
    want, bad = ps.transform(cube)
    assert np.array_equal(np.isneginf(ll), bad)
    _check_phys(ps, phys, want)  # the device API keeps the values of rejected points
    host_ll, _ = ctx.eval_cube(cube)
    assert np.array_equal(ll, host_ll)
    ctx.close()


def test_loglike_callback_writes_physical_values(native):
    ctx = _ctx()
    ps = ParamSpace(OBJECTS, TABLE)
    cube = _cube(ctx.ndims, B=6, seed=13)
    want, bad = ps.transform(cube)
    ll, _ = ctx.eval_cube(cube)
    for b in range(6):
        l1, p1 = ctx.loglike(cube[b])
        _check_phys(ps, p1[None, :], want[b : b + 1])
        assert (l1 == ll[b]) if not bad[b] else np.isneginf(l1)
    ctx.close()
