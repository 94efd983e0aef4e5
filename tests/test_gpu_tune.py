"""Launch shapes and the autotuner on the GPU.

Every candidate shape of the tuner is run through the C ABI on a reduced
version of the headline model (SIE + shear, Sersic bulge, exponential disk,
sky; 96x72 image so that tiles are ragged in both directions; 11x11 PSF;
25-point rule):
  * render images of shapes without a quadrature split are bit-identical
    to the default shape's (per-pixel arithmetic does not depend on the
    tile), convolved images likewise for every convolution tile, and logL
    agrees to 1e-12 relative (only the grouping of FP64 partial sums moves);
  * with a quadrature split (fast mode only) the FP32 quadrature sum is
    reordered: images within 1e-5 relative and logL within the fast-mode
    tolerance of the FP32 oracle (1e-3 + 2e-6 |logL|);
  * exact (default) and strict modes: every candidate (the exact mode's
    quadrature splits included: they sum in the rule's order) gives images
    identical to the oracle-pinned default, and the exact mode's equal the
    strict mode's;
  * the autotuner picks one of its candidates, caches the choice in the
    process and in the LG_TUNE_CACHE file, and its results meet the same
    tolerances; the multi-system kernels likewise.
"""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

import lensed_gb300 as lg
from lensed_gb300 import quadrature, workloads
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
W, H = 96, 72
PLUGINS = ["sie_plus_shear", "sersic", "exponential", "sky"]
TRUTH = np.array([48.7, 36.2, 14.0, 0.75, 40.0, 0.04, -0.02,
                  50.0, 37.5, 4.0, 18.0, 2.5, 0.8, 110.0,
                  50.0, 37.5, 6.0, 18.5, 0.6, 60.0,
                  10.0, -0.0, -0.0])
SPAN = np.array([1, 1, 2, 0.1, 20, 0.03, 0.03, 2, 2, 1, 0.5, 0.5, 0.1, 20, 2, 2, 1, 0.5, 0.1, 20, 1, 0, 0])


def _setup(psf_w=11):
    psf = workloads.psf_gauss_wings(psf_w, 2.0)
    rng = np.random.Generator(np.random.PCG64(11))
    mock = workloads.mock_model(W, H, PLUGINS, TRUTH)
    image = (mock + rng.normal(0, 1.0, mock.shape)).astype(np.float32)
    weight = np.full_like(image, 1.0 / 11.0)
    weight[rng.random(weight.shape) < 0.1] = 0
    lo, hi = TRUTH - SPAN, TRUTH + SPAN
    priors = []
    k = 0
    for p in PLUGINS:
        names = [n for n, *_ in lg.plugin_params(p)]
        d = {}
        for n in names:
            d[n] = repr(float(TRUTH[k])) if SPAN[k] == 0 else f"unif {float(lo[k])!r} {float(hi[k])!r}"
            k += 1
        priors.append(d)
    objs = [(f"o{i}", p, priors[i]) for i, p in enumerate(PLUGINS)]
    cand = TRUTH + (rng.random((16, TRUTH.size)) - 0.5) * SPAN
    return psf, image, weight, objs, cand


def _ctx(objs, image, weight, psf, flags=0, max_batch=16):
    return lg.Context(image, weight, objs, psf=psf, rule="sub5", max_batch=max_batch, flags=flags)


def test_every_fast_candidate_shape(native):
    psf, image, weight, objs, cand = _setup()
    ctx = _ctx(objs, image, weight, psf, flags=lg.LG_FLAG_FAST_MATH)
    p = ctx.to_map_order(cand)
    base_shape = ctx.launch_shape
    base_logl = ctx.eval_batch(p)
    base_model, base_raw, _ = ctx.render(p[0])
    want = Oracle(PLUGINS, W, H, quadrature.rule("sub5"), psf=psf, image=image, weight=weight,
                  precision=32).loglike(cand)
    shapes = lg.tune_candidates(W, H, objs, psf=psf, rule="sub5", flags=lg.LG_FLAG_FAST_MATH)
    assert base_shape in shapes
    for s in shapes:
        ctx.set_launch_shape(**s)
        assert ctx.launch_shape == s
        got = ctx.eval_batch(p)
        model, raw, _ = ctx.render(p[0])
        assert np.all(np.abs(got - want) <= 1e-3 + 2e-6 * np.abs(want)), (s, np.abs(got - want).max())
        if s["qs"] == 1:
            assert np.array_equal(raw, base_raw), s
            assert np.array_equal(model, base_model), s
            assert np.allclose(got, base_logl, rtol=1e-12, atol=0), (s, np.abs(got - base_logl).max())
        else:
            rel = np.abs(raw - base_raw).max() / np.abs(base_raw).max()
            assert rel <= 1e-5, (s, rel)
        print(f"{s}: max|dlogL| vs FP32 oracle {np.abs(got - want).max():.3g}")


@pytest.mark.parametrize("flags", [0, lg.LG_FLAG_STRICT_FP])
def test_every_exact_and_strict_candidate_shape(native, flags):
    psf, image, weight, objs, cand = _setup()
    ctx = _ctx(objs, image, weight, psf, flags=flags)
    p = ctx.to_map_order(cand)
    base_logl = ctx.eval_batch(p)
    base_model, base_raw, base_err = ctx.render(p[0])
    if not flags:
        strict = _ctx(objs, image, weight, psf, flags=lg.LG_FLAG_STRICT_FP)
        s_model, s_raw, s_err = strict.render(p[0])
        assert np.array_equal(base_raw, s_raw) and np.array_equal(base_err, s_err)
        assert np.array_equal(base_model, s_model)
        assert np.allclose(base_logl, strict.eval_batch(p), rtol=1e-12, atol=0)  # FP64 summation grouping
        strict.close()
    shapes = lg.tune_candidates(W, H, objs, psf=psf, rule="sub5", flags=flags)
    assert len(shapes) >= 5
    if not flags:
        assert any(s["qs"] > 1 for s in shapes)  # ordered splits: still identical images
    for s in shapes:
        ctx.set_launch_shape(**s)
        model, raw, err = ctx.render(p[0])
        assert np.array_equal(raw, base_raw) and np.array_equal(err, base_err), s
        assert np.array_equal(model, base_model), s
        assert np.allclose(ctx.eval_batch(p), base_logl, rtol=1e-12, atol=0), s
    with pytest.raises(lg.LensedError):
        ctx.set_launch_shape(qs=2, rppt=1)  # no split of single pixels (exact), no split at all (strict)
    assert ctx.launch_shape == shapes[-1]  # unchanged by the rejected call


def test_autotune_picks_a_candidate_and_caches_it(native):
    psf, image, weight, objs, cand = _setup()
    ctx = _ctx(objs, image, weight, psf, flags=lg.LG_FLAG_AUTOTUNE, max_batch=64)
    rep = ctx.tune_report
    print(rep)
    assert rep.startswith("tuned"), rep
    shapes = lg.tune_candidates(W, H, objs, psf=psf, rule="sub5")
    chosen = ctx.launch_shape
    assert (chosen["rt"], chosen["rppt"], chosen["qs"]) in {(s["rt"], s["rppt"], s["qs"]) for s in shapes}
    assert (chosen["ctx"], chosen["cty"], chosen["cr"]) in {(s["ctx"], s["cty"], s["cr"]) for s in shapes}
    got = ctx.eval_batch(ctx.to_map_order(cand))
    want = Oracle(PLUGINS, W, H, quadrature.rule("sub5"), psf=psf, image=image, weight=weight,
                  precision=32).loglike(cand)
    assert np.all(np.abs(got - want) <= 1e-3)  # the exact mode's tolerance
    again = _ctx(objs, image, weight, psf, flags=lg.LG_FLAG_AUTOTUNE, max_batch=64)
    assert again.tune_report.startswith("cached") and again.launch_shape == chosen
    other = _ctx(objs, image, weight, psf, flags=lg.LG_FLAG_AUTOTUNE, max_batch=32)  # another batch: own entry
    assert other.tune_report.startswith("tuned")


def test_shape_change_after_small_batch_calls(native):
    """A launch-shape change replaces the evaluation module: the graphs
    captured for earlier calls (batches through the host object data
    included) are released with it, and later calls of every batch size
    capture new ones and give the same logL."""
    psf, image, weight, objs, cand = _setup()
    ctx = _ctx(objs, image, weight, psf, max_batch=16)
    p = ctx.to_map_order(cand)
    before = [ctx.eval_batch(p[:1]), ctx.eval_batch(p[:3]), ctx.eval_batch(p)]
    cube = np.full((1, ctx.ndims), 0.4)
    cb, _ = ctx.eval_cube(cube)
    base = ctx.launch_shape
    other = dict(rt=64, rppt=2, qs=1, ctx=32, cty=16, cr=4, pair_rows=0)
    assert other != base
    ctx.set_launch_shape(**other)
    after = [ctx.eval_batch(p[:1]), ctx.eval_batch(p[:3]), ctx.eval_batch(p)]
    ca, _ = ctx.eval_cube(cube)
    for x, y in zip(before, after):
        np.testing.assert_allclose(x, y, rtol=1e-12, atol=0)
    np.testing.assert_allclose(ca, cb, rtol=1e-12, atol=0)
    ctx.set_launch_shape(**base)
    assert np.array_equal(ctx.eval_batch(p[:1]), before[0])


def test_autotune_file_cache_across_processes(native, tmp_path):
    cache = tmp_path / "tune.txt"
    script = textwrap.dedent(f"""
        import sys
        sys.path.insert(0, {ROOT!r})
        sys.path.insert(0, {os.path.join(ROOT, 'tests')!r})
        import lensed_gb300 as lg
        from test_gpu_tune import _setup, _ctx
        psf, image, weight, objs, cand = _setup()
        ctx = _ctx(objs, image, weight, psf, flags=lg.LG_FLAG_AUTOTUNE, max_batch=48)
        print(ctx.tune_report.split()[0], sorted(ctx.launch_shape.items()))
    """)
    env = dict(os.environ, LG_TUNE_CACHE=str(cache))
    runs = [subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True, timeout=300)
            for _ in range(2)]
    for r in runs:
        assert r.returncode == 0, r.stderr
    first, second = (r.stdout.strip().splitlines()[-1] for r in runs)
    assert first.startswith("tuned") and second.startswith("cached"), (first, second)
    assert first.split(" ", 1)[1] == second.split(" ", 1)[1]
    assert len(cache.read_text().splitlines()) == 1


def test_no_psf_and_missing_priors(native):
    _, image, weight, objs, cand = _setup()
    ctx = _ctx(objs, image, weight, None, flags=lg.LG_FLAG_AUTOTUNE)
    assert ctx.tune_report.startswith("tuned")
    want = Oracle(PLUGINS, W, H, quadrature.rule("sub5"), image=image, weight=weight,
                  precision=32).loglike(cand)
    got = ctx.eval_batch(ctx.to_map_order(cand))
    assert np.all(np.abs(got - want) <= 1e-3)
    # without priors there is nothing to draw timing candidates from (the
    # cache key is the evaluation program's, which priors do not change:
    # another batch size keeps this from being a cache hit)
    bare = [(f"o{i}", p, None) for i, p in enumerate(PLUGINS)]
    ctx2 = _ctx(bare, image, weight, None, flags=lg.LG_FLAG_AUTOTUNE, max_batch=24)
    assert ctx2.tune_report.startswith("not tuned"), ctx2.tune_report
    assert np.allclose(ctx2.eval_batch(ctx2.to_map_order(cand)), got, rtol=1e-12, atol=0)


MULTI_RENDER = [(128, 2, 1), (256, 2, 1), (64, 2, 1), (128, 4, 1), (128, 2, 2), (256, 2, 2), (128, 2, 4), (128, 2, 8)]
MULTI_CONV = [(32, 32, 8), (32, 16, 8), (64, 32, 8), (64, 16, 8), (32, 32, 16), (32, 8, 8)]


def test_systems_shapes_and_autotune(native):
    """Fast mode (quadrature splits reorder the sum); the tuned exact
    systems (ordered splits) match the untuned ones bit for bit."""
    syst = workloads.systems(count=4)
    objs = syst[0].objects
    S = lg.Systems([(s.image, s.weight, s.psf, None) for s in syst], objs, capacity=[6] * 4, rule="g3k7",
                   flags=lg.LG_FLAG_FAST_MATH)
    params = []
    for k, s in enumerate(syst):
        c = lg.Context(s.image, s.weight, s.objects, psf=s.psf, rule=s.rule, max_batch=1)
        params.append(c.to_map_order(workloads.draw_candidates(s, 6, seed=k)))
        c.close()
    base = np.concatenate(S.eval(params))
    shapes = [dict(rt=r, rppt=p, qs=q) for r, p, q in MULTI_RENDER] + \
             [dict(ctx=x, cty=y, cr=c) for x, y, c in MULTI_CONV]
    for s in shapes:
        S.set_launch_shape(rt=128, rppt=2, qs=1, ctx=32, cty=32, cr=8)
        S.set_launch_shape(**s)
        got = np.concatenate(S.eval(params))
        if S.launch_shape["qs"] == 1:
            assert np.allclose(got, base, rtol=1e-12, atol=0), (s, np.abs(got - base).max())
        else:
            assert np.all(np.abs(got - base) <= 1e-3 + 2e-6 * np.abs(base)), (s, np.abs(got - base).max())
    T = lg.Systems([(s.image, s.weight, s.psf, None) for s in syst], objs, capacity=[6] * 4, rule="g3k7",
                   flags=lg.LG_FLAG_AUTOTUNE | lg.LG_FLAG_FAST_MATH)
    print(T.tune_report)
    assert T.tune_report.startswith("tuned")
    got = np.concatenate(T.eval(params))
    assert np.all(np.abs(got - base) <= 1e-3 + 2e-6 * np.abs(base))
    E = lg.Systems([(s.image, s.weight, s.psf, None) for s in syst], objs, capacity=[6] * 4, rule="g3k7")
    TE = lg.Systems([(s.image, s.weight, s.psf, None) for s in syst], objs, capacity=[6] * 4, rule="g3k7",
                    flags=lg.LG_FLAG_AUTOTUNE)
    ex = np.concatenate(E.eval(params))
    assert np.allclose(np.concatenate(TE.eval(params)), ex, rtol=1e-12, atol=0)
    with pytest.raises(lg.LensedError):
        S.set_launch_shape(cr=4)  # multi-system units need cr % 8 == 0
