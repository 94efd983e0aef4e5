"""Launch-shape autotuner, host side (no GPU): the candidate shapes a model
gets, their validation, and that every candidate's evaluation module
composes and compiles with NVRTC for sm_103a."""
from concurrent.futures import ThreadPoolExecutor

import pytest

import lensed_gb300 as lg
from lensed_gb300 import workloads

OBJS = [("lens", "sie_plus_shear", None), ("bulge", "sersic", None), ("disk", "exponential", None),
        ("sky", "sky", None)]


def _compile_all(shapes, **kw):
    def one(s):
        return lg.compile_check_shape(96, 72, OBJS, s, **kw)

    with ThreadPoolExecutor(max_workers=8) as ex:
        list(ex.map(one, shapes))


def test_fast_mode_candidates_with_psf_compile(native):
    psf = workloads.psf_gauss_wings(11, 2.0)
    fast = lg.LG_FLAG_FAST_MATH
    shapes = lg.tune_candidates(96, 72, OBJS, psf=psf, rule="sub5", flags=fast)
    render = {(s["rt"], s["rppt"], s["qs"]) for s in shapes}
    conv = {(s["ctx"], s["cty"], s["cr"]) for s in shapes}
    assert (128, 2, 1) in render and any(q > 1 for _, _, q in render)  # quadrature split candidates
    assert len(conv) >= 4 and sum(s["pair_rows"] == 1 for s in shapes) >= 7
    # single-row tiles of four outputs per thread for small batches
    assert any(s["pair_rows"] == 0 and s["cr"] == 4 for s in shapes)
    _compile_all(shapes, psf=psf, rule="sub5", flags=fast)


def test_exact_mode_candidates_pair_rays_and_keep_the_quadrature_order(native):
    """The default (exact) mode: paired rays and paired convolution rows;
    quadrature splits sum the gathered values in the rule's order."""
    psf = workloads.psf_gauss_wings(11, 2.0)
    shapes = lg.tune_candidates(96, 72, OBJS, psf=psf, rule="sub5")
    assert shapes and any(s["qs"] > 1 for s in shapes) and all(s["rppt"] % 2 == 0 for s in shapes if s["qs"] > 1)
    assert sum(s["pair_rows"] == 1 for s in shapes) >= 5
    _compile_all(shapes, psf=psf, rule="sub5")


def test_strict_candidates_keep_the_quadrature_order(native):
    psf = workloads.psf_gauss_wings(11, 2.0)
    shapes = lg.tune_candidates(96, 72, OBJS, psf=psf, rule="sub5", flags=lg.LG_FLAG_STRICT_FP)
    assert shapes and all(s["qs"] == 1 and s["pair_rows"] == 0 for s in shapes)
    _compile_all(shapes, psf=psf, rule="sub5", flags=lg.LG_FLAG_STRICT_FP)


def test_no_psf_candidates_are_render_only(native):
    shapes = lg.tune_candidates(96, 72, OBJS, rule="sub3")
    assert len({(s["ctx"], s["cty"], s["cr"]) for s in shapes}) == 1
    assert len(shapes) >= 5
    _compile_all(shapes, rule="sub3")


@pytest.mark.parametrize("bad,flags,psfw", [
    (dict(qs=2), lg.LG_FLAG_STRICT_FP, 11),    # strict mode keeps the quadrature sum in order
    (dict(qs=2, rppt=1), 0, 11),                # the exact mode splits pixel pairs only
    (dict(qs=3), lg.LG_FLAG_FAST_MATH, 11),     # split of 1, 2, 4 or 8 threads
    (dict(rt=100), 0, 11),                      # whole warps
    (dict(rppt=0), 0, 11),
    (dict(cr=8, ctx=36), 0, 11),                # tile width a multiple of cr
    (dict(pair_rows=1), 0, 51),                 # paired rows only up to 49-pixel PSFs
    (dict(pair_rows=1, cty=63), 0, 11),         # paired tiles have an even height
    (dict(ctx=256, cr=4, cty=64), 0, 11),       # 2048 threads per block
])
def test_invalid_shapes_are_rejected(native, bad, flags, psfw):
    psf = workloads.psf_gauss_wings(psfw, 2.0)
    base = dict(rt=128, rppt=2, qs=1, ctx=32, cty=32, cr=8, pair_rows=0)
    base.update(bad)
    with pytest.raises(lg.LensedError) as e:
        lg.compile_check_shape(96, 72, OBJS, base, psf=psf, rule="sub5", flags=flags)
    assert e.value.code == -1  # LG_ERR_INPUT
