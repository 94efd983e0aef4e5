"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

The FP32 reference semantics is IEEE single-precision arithmetic in the
reference's operation order with elementary functions evaluated in double
and rounded once (oracle math="cr").  set_params always follows it on the
GPU.  Three evaluation modes:

* default (exact): ray pairs, no contraction, correctly rounded functions
  (single-precision double-word arithmetic with a rounding test, double
  only where the test cannot decide).  It must give the strict mode's
  images bit for bit, and match the oracle as strict does;
* strict (LG_FLAG_STRICT_FP): one ray at a time, functions in double.
  Images within 2 ulp of the oracle (1.2e-7 relative; identical except for
  rare double-rounding coincidences between CUDA's and the C library's
  double functions) and |dlogL| <= 1e-3 absolute (measured: 1e-10, the
  FP64 summation order);
* fast (LG_FLAG_FAST_MATH): FMA contraction and hardware-approximate
  functions per ray (within a few ulp); its tolerances:
  - model images: relative error <= 1e-5 on pixels above 1e-6 of the peak,
    absolute error <= 1e-6 * peak below that floor.  Where the FP32 oracle
    is itself further than 1e-5 from the FP64 oracle (ill-conditioned
    profiles, e.g. the r^(1/4) cusp of de Vaucouleurs, whose gradient
    amplifies last-bit differences of the ray positions), the bound is three
    times that FP32 error, and the GPU image must be as close to FP64 as
    that bound;
  - logL: |logL_gpu - logL_oracle32| <= 1e-3 + 2e-6 |logL| (the ulp-level
    differences of the per-ray functions add up coherently for candidates
    far from the data, and the Sersic profile exp(log0 - exp(u)) amplifies
    a last-bit difference of the inner exp by its value).
The FP32 paths' distance to the FP64 oracle is reported, not bounded
tighter than the FP32 budget.
"""
import os

import numpy as np
import pytest

import lensed_gb300 as lg
from lensed_gb300 import quadrature, workloads
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

IMG_REL, LOGL_ABS, LOGL_REL = 1e-5, 1e-3, 2e-6
EXACT, STRICT, FAST = 0, lg.LG_FLAG_STRICT_FP, lg.LG_FLAG_FAST_MATH


def logl_tol(ref, flags=FAST):
    """|dlogL| bound: 1e-3 absolute for the exact and strict modes; the fast
    mode's widened bound."""
    if not flags & FAST:
        return np.full_like(np.asarray(ref, np.float64), LOGL_ABS)
    return LOGL_ABS + LOGL_REL * np.abs(ref)


def assert_bitwise_close(got, want, what=""):
    """The exact and strict modes: at least 99.9% of the pixels identical to
    the oracle's, the others within 2 ulp."""
    want = np.asarray(want).astype(np.float32)
    same = got == want
    rel = np.abs(got.astype(np.float64) - want) / np.maximum(np.abs(want.astype(np.float64)), 1e-30)
    assert rel.max() <= 2.4e-7 and same.mean() >= 0.999, (what, rel.max(), same.mean())


def image_err(got, want):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    peak = np.abs(want).max()
    big = np.abs(want) > 1e-6 * peak
    rel = (np.abs(got - want)[big] / np.abs(want[big])).max() if big.any() else 0.0
    small = np.abs(got - want)[~big].max() / peak if (~big).any() else 0.0
    return rel, small


def assert_image_close(got, want, what="", want64=None):
    tol = IMG_REL
    if want64 is not None:
        tol = max(IMG_REL, 3 * image_err(want, want64)[0])
        rel64, _ = image_err(got, want64)
        assert rel64 <= tol, (what, "vs FP64", rel64, tol)
    rel, small = image_err(got, want)
    assert rel <= tol and small <= 1e-6, (what, rel, small, tol)


PLUGIN_CASES = [
    (["sis", "sersic"], [20.3, 18.7, 8.0] + [21.0, 18.0, 3.0, -2.0, 1.5, 0.8, 20.0]),
    (["sis_plus_shear", "sersic"], [20.3, 18.7, 8.0, 0.05, -0.03] + [21.0, 18.0, 3.0, -2.0, 1.5, 0.8, 20.0]),
    (["nsis", "exponential"], [20.3, 18.7, 8.0, 1.5] + [21.0, 18.0, 3.0, -2.0, 0.8, 20.0]),
    (["sie", "devauc"], [20.3, 18.7, 8.0, 0.7, 35.0] + [21.0, 18.0, 3.0, -2.0, 0.8, 20.0]),
    (["sie_plus_shear", "gauss"], [20.3, 18.7, 8.0, 0.7, 35.0, 0.05, -0.03] + [21.0, 18.0, 3.0, -2.0, 0.8, 20.0]),
    (["nsie", "sersic_old"], [20.3, 18.7, 8.0, 1.2, 0.7, 35.0] + [21.0, 18.0, 3.0, -2.0, 2.5, 0.8, 20.0]),
    (["point_mass", "sersic"], [20.3, 18.7, 6.0] + [21.0, 18.0, 3.0, -2.0, 1.5, 0.8, 20.0]),
    (["epl", "sersic"], [20.3, 18.7, 8.0, 0.8, 0.7, 35.0] + [21.0, 18.0, 3.0, -2.0, 1.5, 0.8, 20.0]),
    (["epl_plus_shear", "sersic"], [20.3, 18.7, 8.0, 1.2, 0.7, 35.0, 0.05, -0.03] + [21.0, 18.0, 3.0, -2.0, 1.5, 0.8, 20.0]),
    (["sky"], [10.0, 0.3, -0.2]),
    (["sersic", "sie", "sersic", "sky"], [15.0, 25.0, 2.0, -1.0, 3.0, 0.6, 100.0, 20.3, 18.7, 8.0, 0.7, 35.0,
                                          21.0, 18.0, 3.0, -2.0, 1.5, 0.8, 20.0, 10.0, 0.1, 0.2]),
]


def make_ctx(plugins, W, H, psf=None, rule="g3k7", image=None, weight=None, pcs=None, max_batch=64, flags=0,
             priors=None):
    if image is None:
        image = np.zeros((H, W), np.float32)
    if weight is None:
        weight = np.ones((H, W), np.float32)
    objs = [(f"o{i}", p, None if priors is None else priors[i]) for i, p in enumerate(plugins)]
    return lg.Context(image, weight, objs, psf=psf, rule=rule, pcs=pcs, max_batch=max_batch, flags=flags)


@pytest.mark.parametrize("case", range(len(PLUGIN_CASES)))
def test_fast_render_matches_oracle_per_plugin(native, case):
    plugins, params = PLUGIN_CASES[case]
    W, H = 41, 37  # non-square, odd: catches index mix-ups
    pcs = (2.0, -1.0, 1.0, 1.0)
    ctx = make_ctx(plugins, W, H, rule="gm75", pcs=pcs, flags=FAST)
    model, raw, err = ctx.render(ctx.to_map_order(params))
    o = Oracle(plugins, W, H, quadrature.rule("gm75"), pcs=pcs, precision=32)
    v, e, _ = o.render(params)
    v64 = Oracle(plugins, W, H, quadrature.rule("gm75"), pcs=pcs, precision=64).render(params)[0]
    assert_image_close(raw, v, plugins, want64=v64)
    assert np.array_equal(model, raw)  # no PSF: the model is the raw render
    tol = max(IMG_REL, 3 * image_err(v, v64)[0])
    assert np.abs(err - e).max() <= tol * np.abs(v).max() + 1e-7, plugins


@pytest.mark.parametrize("case", range(len(PLUGIN_CASES)))
def test_exact_and_strict_render_match_oracle_bitwise(native, case):
    """The exact mode's images equal the strict mode's bit for bit (value,
    error and model images), and both match the oracle to the last bit."""
    plugins, params = PLUGIN_CASES[case]
    W, H = 41, 37
    pcs = (2.0, -1.0, 1.0, 1.0)
    v, e, _ = Oracle(plugins, W, H, quadrature.rule("gm75"), pcs=pcs, precision=32).render(params)
    out = {}
    for flags, name in ((EXACT, "exact"), (STRICT, "strict")):
        ctx = make_ctx(plugins, W, H, rule="gm75", pcs=pcs, flags=flags)
        _, raw, err = ctx.render(ctx.to_map_order(params))
        same = raw == v.astype(np.float32)
        print(f"{name} {plugins}: {100 * same.mean():.4f}% identical pixels")
        assert_bitwise_close(raw, v, (name, plugins))
        out[name] = (raw, err)
        ctx.close()
    assert np.array_equal(out["exact"][0], out["strict"][0]), plugins
    assert np.array_equal(out["exact"][1], out["strict"][1]), plugins


def test_reference_images_on_gpu(native, golden):
    rule = quadrature.rule("g3k7")
    for case in [str(c) for c in golden["cases"]]:
        plugins = [str(p) for p in golden[f"{case}__plugins"]]
        params = golden[f"{case}__params"]
        ctx = make_ctx(plugins, 100, 100, rule="g3k7")
        _, raw, _ = ctx.render(ctx.to_map_order(params))
        want = Oracle(plugins, 100, 100, rule, precision=32).render(params)[0]
        assert_image_close(raw, want, case)
        ref = golden[f"{case}__image"].astype(np.float64)
        big = np.abs(ref) > 1e-6 * np.abs(ref).max()
        assert (np.abs(raw - ref)[big] / np.abs(ref[big])).max() <= 2e-4, case
        ctx.close()


@pytest.mark.parametrize("psf_size", [7, 8, 15, 49, 51])
@pytest.mark.parametrize("flags", [EXACT, STRICT, FAST])
def test_psf_convolution_matches_oracle(native, psf_size, flags):
    """Paired-row convolution (fast and exact modes, PSF width <= 49) and
    the single-row kernel (strict mode, wider PSFs), on images smaller than
    the PSF too."""
    plugins, params = PLUGIN_CASES[4]
    W, H = (45, 52) if psf_size < 40 else (40, 70)
    psf = workloads.psf_gauss_wings(psf_size, 2.0)
    if psf_size == 8:
        psf = psf[:, :7].copy()  # even height, odd width: one-axis half-pixel shift
    ctx = make_ctx(plugins, W, H, psf=psf, rule="sub2", flags=flags)
    model, raw, _ = ctx.render(ctx.to_map_order(params))
    o = Oracle(plugins, W, H, quadrature.rule("sub2"), psf=psf, precision=32)
    v, _, c = o.render(params)
    assert_image_close(raw, v, "raw")
    assert_image_close(model, c, "convolved")
    if not flags & FAST:
        assert_bitwise_close(raw, v, "raw")
        assert_bitwise_close(model, c, "convolved")


@pytest.mark.parametrize("W,H,psf_size", [(5, 3, 7), (45, 52, 101), (20, 17, 1), (24, 30, 71), (33, 1, 9)])
@pytest.mark.parametrize("flags", [EXACT, STRICT, FAST])
def test_convolution_edge_sizes(native, W, H, psf_size, flags):
    """Images smaller than one tile, the largest PSF (101 x 101), a 1 x 1
    PSF, PSFs larger than the image in both directions and a one-row image:
    the clamp-to-edge convolution equals the oracle's, and the logL too."""
    plugins, params = PLUGIN_CASES[4]
    params = list(params)
    params[0], params[1] = (W + 1) / 2, (H + 1) / 2
    psf = workloads.psf_gauss_wings(psf_size, 2.0) if psf_size > 1 else np.ones((1, 1), np.float32)
    rng = np.random.Generator(np.random.PCG64(psf_size))
    image = rng.normal(10.0, 1.0, (H, W)).astype(np.float32)
    weight = rng.uniform(0.5, 1.5, (H, W)).astype(np.float32)
    ctx = make_ctx(plugins, W, H, psf=psf, rule="sub2", flags=flags, image=image, weight=weight)
    p = ctx.to_map_order(params)
    model, raw, _ = ctx.render(p)
    o = Oracle(plugins, W, H, quadrature.rule("sub2"), psf=psf, image=image, weight=weight, precision=32)
    v, _, c = o.render(params)
    assert_image_close(raw, v, "raw")
    assert_image_close(model, c, "convolved")
    got = ctx.eval_batch(p[None, :])
    want = o.loglike(np.asarray(params)[None, :])
    assert np.all(np.abs(got - want) <= logl_tol(want, flags)), (got, want)


def test_fully_masked_image_and_oversized_psf(native):
    """All weights zero: chi^2 = 0, logL = 0 for every candidate; a PSF above
    the 101 x 101 limit is refused with a status, not a crash."""
    plugins, params = PLUGIN_CASES[4]
    W, H = 40, 30
    ctx = make_ctx(plugins, W, H, psf=workloads.psf_gauss_wings(9, 2.0), rule="sub2",
                   weight=np.zeros((H, W), np.float32))
    assert ctx.masked == W * H
    got = ctx.eval_batch(np.tile(ctx.to_map_order(params), (5, 1)))
    assert np.all(got == 0.0)
    with pytest.raises(lg.LensedError):
        make_ctx(plugins, W, H, psf=workloads.psf_gauss_wings(103, 2.0), rule="sub2")


def _loglike_case(system, B, seed=0, flags=EXACT):
    ctx = lg.Context(system.image, system.weight, system.objects, psf=system.psf, rule=system.rule,
                     max_batch=max(B, 8), flags=flags)
    cand = workloads.draw_candidates(system, B, seed=seed)
    got = ctx.eval_batch(ctx.to_map_order(cand))
    o32 = Oracle(system.plugins, system.width, system.height, quadrature.rule(system.rule), psf=system.psf,
                 image=system.image, weight=system.weight, precision=32, threads=16)
    o64 = Oracle(system.plugins, system.width, system.height, quadrature.rule(system.rule), psf=system.psf,
                 image=system.image, weight=system.weight, precision=64, threads=16)
    want32, want64 = o32.loglike(cand), o64.loglike(cand)
    return ctx, cand, got, want32, want64


def _report(name, got, w32, w64):
    d32 = np.abs(got - w32)
    print(f"{name}: |dlogL| vs FP32 oracle max {d32.max():.3g} (per candidate {np.array2string(d32, precision=2)}), "
          f"vs FP64 oracle max {np.abs(got - w64).max():.3g}, FP32 oracle vs FP64 max {np.abs(w32 - w64).max():.3g}")
    return d32


@pytest.mark.parametrize("flags", [EXACT, FAST])
def test_loglike_small_workload(native, flags):
    ctx, cand, got, w32, w64 = _loglike_case(workloads.small(), 16, flags=flags)
    d32 = _report(f"small {'fast' if flags else 'exact'}", got, w32, w64)
    assert np.all(d32 <= logl_tol(w32, flags))
    # closer to the FP32 reference than FP32 is to FP64
    assert np.abs(got - w32).max() < 0.5 * np.abs(w32 - w64).max()


@pytest.mark.parametrize("flags", [EXACT, FAST])
def test_loglike_config2_full_size(native, flags):
    """256^2, SIE+shear, bulge + disk + sky, 25x25 PSF, 25-point rule, 10% mask."""
    ctx, cand, got, w32, w64 = _loglike_case(workloads.config2(), 8, flags=flags)
    d32 = _report(f"config2 {'fast' if flags else 'exact'}", got, w32, w64)
    assert np.all(d32 <= logl_tol(w32, flags))
    assert np.abs(got - w32).max() < 0.5 * np.abs(w32 - w64).max()
    assert ctx.masked == int((ctx._weight == 0).sum())


def test_loglike_config2_exact_many_candidates(native):
    """The benchmarked configuration in the default (exact) mode over 256
    seeded prior draws: |dlogL| <= 1e-3 absolute against the FP32 oracle for
    every candidate (the benchmark spec's bound; measured about 1e-10)."""
    ctx, cand, got, w32, w64 = _loglike_case(workloads.config2(), 256, seed=12)
    d = np.abs(got - w32)
    print(f"config2 exact, 256 candidates: |dlogL| max {d.max():.3g}, median {np.median(d):.3g}; "
          f"|logL| {np.abs(w32).min():.3g} to {np.abs(w32).max():.3g}; vs FP64 max {np.abs(got - w64).max():.3g}")
    assert d.max() <= LOGL_ABS


def test_loglike_large_workload_full_size(native):
    """The large configuration at full size: 1024^2 at 0.02"/px, EPL+shear +
    NSIE satellite + point mass, two Sersic sources and a Gaussian clump,
    sky, 41x41 PSF, 49-point g3k7 rule.  Two candidates against the FP32
    oracle (tolerance as everywhere) with the error against the all-FP64
    oracle stated for each, in the exact, strict and fast modes."""
    s = workloads.large()
    cand = workloads.draw_candidates(s, 2, seed=3)
    threads = max(16, os.cpu_count() or 1)
    o32 = Oracle(s.plugins, s.width, s.height, quadrature.rule(s.rule), psf=s.psf, image=s.image, weight=s.weight,
                 precision=32, threads=threads)
    o64 = Oracle(s.plugins, s.width, s.height, quadrature.rule(s.rule), psf=s.psf, image=s.image, weight=s.weight,
                 precision=64, threads=threads)
    w32, w64 = o32.loglike(cand), o64.loglike(cand)
    for flags, name in ((EXACT, "large exact"), (STRICT, "large strict"), (FAST, "large fast")):
        ctx = lg.Context(s.image, s.weight, s.objects, psf=s.psf, rule=s.rule, max_batch=2, flags=flags)
        got = ctx.eval_batch(ctx.to_map_order(cand))
        d32 = _report(name, got, w32, w64)
        print(f"{name}: relative error vs the FP64 oracle {np.array2string(np.abs(got - w64) / np.abs(w64), precision=2)}")
        assert np.all(d32 <= logl_tol(w32, flags))
        ctx.close()


def test_loglike_config2_fast_ieee_division(native):
    """Fast mode with IEEE division and square root (LG_FLAG_IEEE_DIV)."""
    s = workloads.config2()
    ctx = lg.Context(s.image, s.weight, s.objects, psf=s.psf, rule=s.rule, max_batch=8,
                     flags=FAST | lg.LG_FLAG_IEEE_DIV)
    cand = workloads.draw_candidates(s, 8, seed=0)
    got = ctx.eval_batch(ctx.to_map_order(cand))
    o = Oracle(s.plugins, s.width, s.height, quadrature.rule(s.rule), psf=s.psf, image=s.image, weight=s.weight,
               precision=32, threads=16)
    want = o.loglike(cand)
    d = _report("config2 fast ieee-div", got, want, want)
    assert np.all(d <= logl_tol(want))


@pytest.mark.parametrize("name", ["small", "config2"])
def test_loglike_exact_equals_strict(native, name):
    """The exact and strict modes give the same images, so their logL differ
    only by the grouping of the FP64 partial sums of their launch shapes
    (about 1e-15 relative), and lie within 1e-6 of the oracle's."""
    s = getattr(workloads, name)()
    cand = workloads.draw_candidates(s, 8, seed=5)
    o = Oracle(s.plugins, s.width, s.height, quadrature.rule(s.rule), psf=s.psf, image=s.image, weight=s.weight,
               precision=32, threads=16)
    want = o.loglike(cand)
    got = {}
    for flags, mode in ((EXACT, "exact"), (STRICT, "strict")):
        ctx = lg.Context(s.image, s.weight, s.objects, psf=s.psf, rule=s.rule, max_batch=8, flags=flags)
        got[mode] = ctx.eval_batch(ctx.to_map_order(cand))
        d = _report(f"{name} {mode}", got[mode], want, want)
        assert d.max() <= 1e-6
        ctx.close()
    assert np.allclose(got["exact"], got["strict"], rtol=1e-12, atol=0)


def test_batch_equals_single_and_is_deterministic(native):
    s = workloads.config2()
    ctx = lg.Context(s.image, s.weight, s.objects, psf=s.psf, rule=s.rule, max_batch=64)
    cand = ctx.to_map_order(workloads.draw_candidates(s, 64, seed=3))
    a = ctx.eval_batch(cand)
    b = ctx.eval_batch(cand)
    assert np.array_equal(a, b)
    single = np.array([ctx.eval_batch(cand[i:i + 1])[0] for i in range(0, 64, 9)])
    assert np.array_equal(single, a[::9])
    rev = ctx.eval_batch(cand[::-1].copy())
    assert np.array_equal(rev[::-1], a)


def test_device_entry_points_wait_for_the_legacy_stream(native):
    """Device buffers that a framework writes with kernels queued on the
    legacy default stream (PyTorch's default) are touched only after those
    kernels when the call runs on the context's stream: the profile and the
    NULL-stream device entry point agree with the host path, and the fill of
    the logL buffer does not land after the library's results."""
    torch = pytest.importorskip("torch")
    s = workloads.config2()
    B = 1024
    ctx = lg.Context(s.image, s.weight, s.objects, psf=s.psf, rule=s.rule, max_batch=B)
    cand = ctx.to_map_order(workloads.draw_candidates(s, B, seed=7))
    want = ctx.eval_batch(cand)
    torch.cuda.synchronize()
    assert cand.flags["C_CONTIGUOUS"]
    d_params = torch.tensor(cand, dtype=torch.float64, device="cuda")
    d_logL = torch.full((B,), 7.0, dtype=torch.float64, device="cuda")
    ctx.profile(d_params.data_ptr(), B, d_logL.data_ptr())
    assert np.array_equal(d_logL.cpu().numpy(), want)
    d_params2 = torch.tensor(cand[::-1].copy(), dtype=torch.float64, device="cuda")
    d_logL2 = torch.full((B,), 7.0, dtype=torch.float64, device="cuda")
    ctx.eval_batch_device(d_params2.data_ptr(), B, d_logL2.data_ptr())
    torch.cuda.synchronize()
    ctx.eval_batch(cand[:1])  # synchronises the context's stream
    assert np.array_equal(d_logL2.cpu().numpy(), want[::-1])


def test_device_calls_on_different_streams_are_ordered(native):
    """Calls on one context made on different caller streams share its
    scratch; the library orders them, so back-to-back calls on two streams
    (no synchronisation between them) each return their own batch's logL."""
    torch = pytest.importorskip("torch")
    s = workloads.config2()
    B = 256
    ctx = lg.Context(s.image, s.weight, s.objects, psf=s.psf, rule=s.rule, max_batch=B)
    cand = ctx.to_map_order(workloads.draw_candidates(s, 2 * B, seed=17))
    want = ctx.eval_batch(cand[:B]), ctx.eval_batch(cand[B:])
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    d_par = [torch.tensor(cand[:B], device="cuda"), torch.tensor(cand[B:], device="cuda")]
    d_out = [torch.full((B,), 7.0, dtype=torch.float64, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    for rep in range(3):
        for k in range(2):
            ctx.eval_batch_device(d_par[k].data_ptr(), B, d_out[k].data_ptr(), streams[k].cuda_stream)
    torch.cuda.synchronize()
    for k in range(2):
        assert np.array_equal(d_out[k].cpu().numpy(), want[k]), k
    ctx.close()


def test_graph_and_direct_launch_agree(native):
    s = workloads.small()
    cand = workloads.draw_candidates(s, 32, seed=4)
    a = lg.Context(s.image, s.weight, s.objects, rule=s.rule, max_batch=32)
    b = lg.Context(s.image, s.weight, s.objects, rule=s.rule, max_batch=32, flags=lg.LG_FLAG_NO_GRAPH)
    assert np.array_equal(a.eval_batch(a.to_map_order(cand)), b.eval_batch(b.to_map_order(cand)))


def test_image_plane_prior_parity(native):
    W = H = 48
    psf = None
    plugins = ["sie", "sersic"]
    params = [24.3, 23.8, 9.0, 0.75, 40.0, 14.0, 30.0, 2.0, -1.0, 2.0, 0.8, 30.0]
    priors = [{"x": "unif 20 28", "y": "unif 20 28", "r": "unif 5 12", "q": "unif 0.5 0.95", "pa": "unif 0 180"},
              {"x": "image unif 10 20", "y": "image unif 25 35", "r": "unif 1 3", "mag": "unif -3 0",
               "n": "unif 1 4", "q": "unif 0.5 1", "pa": "unif 0 180"}]
    ctx = make_ctx(plugins, W, H, psf=psf, rule="sub3", priors=priors)
    _, raw, _ = ctx.render(ctx.to_map_order(params))
    o = Oracle([("sie", 0), ("sersic", 1)], W, H, quadrature.rule("sub3"), precision=32)
    assert_image_close(raw, o.render(params)[0], "ipp")


def test_host_set_params_match_the_set_module(native):
    """Batches of up to 4 candidates through the host API take their object
    data (and, from the unit cube, the prior transform) from the host: the
    logL of one candidate at a time equals the batched (set_params kernel)
    logL bit for bit, in every mode and with image-plane priors (deflected
    through the lens on the host)."""
    s = workloads.config2()
    for flags in (EXACT, STRICT, FAST):
        ctx = lg.Context(s.image, s.weight, s.objects, psf=s.psf, rule=s.rule, max_batch=16, flags=flags)
        assert ctx.host_set
        cand = ctx.to_map_order(workloads.draw_candidates(s, 16, seed=21))
        batch = ctx.eval_batch(cand)
        for B in (1, 2, 3, 4):
            part = np.concatenate([ctx.eval_batch(cand[i:i + B]) for i in range(0, 16 - 16 % B, B)])
            assert np.array_equal(part, batch[:len(part)]), (flags, B)
        cube = np.random.Generator(np.random.PCG64(5)).random((8, ctx.ndims))
        ll8, ph8 = ctx.eval_cube(cube)
        for b in range(8):
            l1, p1 = ctx.loglike(cube[b])
            assert l1 == ll8[b] and np.array_equal(p1, ph8[b])
        ctx.close()
    W = H = 48
    priors = [{"x": "unif 20 28", "y": "unif 20 28", "r": "unif 5 12", "q": "unif 0.5 0.95", "pa": "unif 0 180"},
              {"x": "image unif 10 20", "y": "image unif 25 35", "r": "unif 1 3", "mag": "unif -3 0",
               "n": "unif 1 4", "q": "unif 0.5 1", "pa": "unif 0 180"}]
    ctx = make_ctx(["sie", "sersic"], W, H, psf=None, rule="sub3", priors=priors, max_batch=8)
    assert ctx.host_set
    cube = np.random.Generator(np.random.PCG64(6)).random((8, ctx.ndims))
    ll8, ph8 = ctx.eval_cube(cube)
    single = np.array([ctx.eval_cube(cube[b:b + 1])[0][0] for b in range(8)])
    assert np.array_equal(single, ll8)
    ctx.close()
    # every built-in plugin: one candidate at a time against a batch of 8
    rng = np.random.Generator(np.random.PCG64(7))
    for plugins, params in PLUGIN_CASES:
        ctx = make_ctx(plugins, 41, 37, rule="sub3", image=np.full((37, 41), 3.0, np.float32), max_batch=8)
        assert ctx.host_set, plugins
        P = np.tile(ctx.to_map_order(np.array(params)), (8, 1)) * (1 + 0.02 * rng.standard_normal((8, len(params))))
        batch = ctx.eval_batch(P)
        single = np.array([ctx.eval_batch(P[b:b + 1])[0] for b in range(8)])
        assert np.array_equal(single, batch), plugins
        ctx.close()


def test_host_set_params_on_many_prior_draws(native):
    """10^4 unit-cube draws of the benchmarked model: small batches (object
    data and prior transform on the host, the C library's double functions)
    against the batched path (set_params kernel, CUDA's double functions).
    The two round each elementary function's double value to float, so they
    can differ only where that value lies within about 2^-52 of a float
    rounding boundary; the test counts such candidates (expected none)."""
    s = workloads.config2()
    ctx = lg.Context(s.image, s.weight, s.objects, psf=s.psf, rule=s.rule, max_batch=1024)
    assert ctx.host_set
    cube = np.random.Generator(np.random.PCG64(31)).random((10000, ctx.ndims))
    batch = np.concatenate([ctx.eval_cube(cube[i:i + 1024])[0] for i in range(0, 10000, 1024)])
    small = np.concatenate([ctx.eval_cube(cube[i:i + 4])[0] for i in range(0, 10000, 4)])
    same = (batch == small) | (np.isnan(batch) & np.isnan(small))
    print(f"host vs kernel set_params: {int((~same).sum())} of 10000 prior draws differ")
    assert same.all()
    ctx.close()


def test_cube_transform_and_reference_callback(native):
    s = workloads.small()
    ctx = lg.Context(s.image, s.weight, s.objects, rule=s.rule, max_batch=16)
    rng = np.random.Generator(np.random.PCG64(9))
    cube = rng.random(size=(5, ctx.ndims))
    ll, phys = ctx.eval_cube(cube)
    direct = ctx.eval_batch(phys)
    assert np.array_equal(ll, direct)
    l1, p1 = ctx.loglike(cube[0])
    assert l1 == ll[0] and np.array_equal(p1, phys[0])
    # derived (fixed) parameters sit after the free ones
    assert ctx.ndims == ctx.npars - 2


def test_bad_calls_return_status_and_context_survives(native):
    import ctypes as C

    s = workloads.small()
    ctx = lg.Context(s.image, s.weight, s.objects, rule=s.rule, max_batch=4)
    cand = np.ascontiguousarray(ctx.to_map_order(workloads.draw_candidates(s, 5, seed=1)))
    out = np.zeros(5)
    dp = C.POINTER(C.c_double)
    rc = lg.lib().lg_eval_batch(ctx.h, cand.ctypes.data_as(dp), 5, out.ctypes.data_as(dp))
    assert rc == -1 and b"max_batch" in lg.lib().lg_last_error(ctx.h)
    ok = ctx.eval_batch(cand[:4])
    assert np.all(np.isfinite(ok))


def test_non_finite_parameters_follow_the_reference(native):
    """A non-finite lens deflection sends the ray away (src/kernel.c:86-91);
    a NaN source parameter gives a NaN likelihood, as on the CPU."""
    s = workloads.small()
    ctx = lg.Context(s.image, s.weight, s.objects, rule=s.rule, max_batch=4)
    o = Oracle(s.plugins, s.width, s.height, quadrature.rule(s.rule), image=s.image, weight=s.weight,
               precision=32, threads=16)
    p = np.tile(s.truth, (2, 1))
    p[0, 0] = np.nan          # lens x
    p[1, 8] = np.nan          # source magnitude
    got = ctx.eval_batch(ctx.to_map_order(p))
    want = o.loglike(p)
    assert np.isfinite(got[0]) and abs(got[0] - want[0]) <= logl_tol(want[0], EXACT)
    assert np.isnan(got[1]) and np.isnan(want[1])
