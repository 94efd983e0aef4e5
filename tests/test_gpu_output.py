"""The dumper's output layers on the GPU (src/nested.c:175-257) against the
oracle, and the FITS file written from them.

* The layer arithmetic (RES, ERR, WHT, PVL) is checked bit for bit against
  the oracle's restatement applied to the GPU's own render; the p-value is
  a double erfc rounded to float, so it may differ from the host's libm in
  the last float bit (allowed: 2 ulp).
* The rendered layers (IMG, RAW) are checked against the FP32 oracle's
  render with the model-image tolerance of the likelihood path (relative
  1e-5 above 1e-6 of the peak, or three times the FP32 oracle's own
  distance to the FP64 oracle where the model is ill-conditioned) and bit
  for bit against lg_render.
"""
import numpy as np
import pytest

import lensed_gb300 as lg
from lensed_gb300 import fits, quadrature
from oracle.oracle import DUMP_NAMES, Oracle, dump_layers
from test_gpu_parity import assert_image_close

pytestmark = pytest.mark.gpu

PLUGINS = ["sie_plus_shear", "sersic", "sky"]
PARAMS = [20.3, 18.7, 8.0, 0.7, 35.0, 0.05, -0.03] + [21.0, 18.0, 3.0, -2.0, 1.5, 0.8, 20.0] + [0.5, 0.01, -0.02]


def _case(psf: bool, seed=5, W=48, H=40):
    rng = np.random.default_rng(seed)
    image = rng.normal(5.0, 1.0, size=(H, W)).astype(np.float32)
    weight = rng.uniform(0.5, 2.0, size=(H, W)).astype(np.float32)
    weight[rng.random((H, W)) < 0.1] = 0.0  # masked pixels
    p = None
    if psf:
        y, x = np.mgrid[-3:4, -2:3]
        p = np.exp(-(x**2 + y**2) / 3.0).astype(np.float32)
        p /= p.sum()
    return image, weight, p


def _ulps(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b)


@pytest.mark.parametrize("psf", [False, True])
@pytest.mark.parametrize("flags", [0, lg.LG_FLAG_STRICT_FP])
def test_dump_layers_match_oracle(native, psf, flags):
    image, weight, p = _case(psf)
    H, W = image.shape
    objs = [(f"o{i}", n, None) for i, n in enumerate(PLUGINS)]
    ctx = lg.Context(image, weight, objs, psf=p, rule="gm75", max_batch=4, flags=flags)
    mp = ctx.to_map_order(PARAMS)
    L = ctx.dump(mp)
    assert list(L) == list(DUMP_NAMES)
    model, raw, err = ctx.render(mp)
    assert np.array_equal(L["IMG"], model) and np.array_equal(L["RAW"], raw)
    assert np.array_equal(L["WHT"], weight)

    want = dump_layers(image, weight, model, raw, err)
    for name in ("RES", "ERR"):
        assert np.array_equal(L[name], want[name], equal_nan=True), name
    assert _ulps(L["PVL"], want["PVL"]).max() <= 2

    rule = quadrature.rule("gm75")
    renders = [Oracle(PLUGINS, W, H, rule, psf=p, precision=prec).render(PARAMS) for prec in (32, 64)]
    ref32, ref64 = [(c if psf else v) for v, e, c in renders]
    assert_image_close(L["IMG"], ref32, "IMG", want64=ref64)
    assert_image_close(L["RAW"], renders[0][0], "RAW", want64=renders[1][0])
    # residuals: absolute error within the model's
    peak = np.abs(ref32).max()
    assert np.abs(L["RES"] - (image - ref32)).max() <= 1e-4 * peak + 1e-6 * np.abs(image).max()
    ctx.close()


def test_write_output_file(native, tmp_path):
    image, weight, p = _case(True, seed=9)
    objs = [(f"o{i}", n, None) for i, n in enumerate(PLUGINS)]
    ctx = lg.Context(image, weight, objs, psf=p, rule="g3k7", max_batch=4)
    mp = ctx.to_map_order(PARAMS)
    path = str(tmp_path / "lensed.fits")
    ctx.write_output(mp, path)
    L = ctx.dump(mp)
    hdus = fits.read_hdus(path)
    assert [h.name for h in hdus[1:]] == list(DUMP_NAMES)
    for h in hdus[1:]:
        assert h.data.shape == image.shape
        assert np.array_equal(h.data.astype(np.float32).view(np.uint32), L[h.name].view(np.uint32)), h.name
    ctx.close()
