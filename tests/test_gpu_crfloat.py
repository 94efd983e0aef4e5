"""The correctly rounded exp, log, atan and atanh of the exact evaluation
modules on the GPU, as ray pairs (f32x2 instructions, rcp.approx
estimates), and the EPL lens's sin, cos, pow and atan2 one value at a time
(pow with sixteen fixed exponents and with a second argument derived from
the first, atan2 likewise): for every one of the 2^32 float inputs, paired
with an unrelated second input (so that the two lanes take different paths
and table entries), the result equals the function evaluated in double on the
device and rounded once (NaN matches NaN) -- the strict modules' per-ray
semantics, which the exact modules must reproduce bit for bit.  The count
is over both lanes; the double evaluation itself is within 1-2 double ulp,
so a handful of inputs whose exact value lies within about 2^-51 of a float
rounding boundary could differ without either side being wrong: the test
allows none, and reports any."""
import ctypes as C

import numpy as np
import pytest

import lensed_gb300 as lg

pytestmark = pytest.mark.gpu


def sweep(fn, lo=0, hi=1 << 32):
    bad = C.c_ulonglong()
    first = (C.c_uint * 8)()
    rc = lg.lib().lg_probe_crf_sweep(0, fn, C.c_ulonglong(lo), C.c_ulonglong(hi), C.byref(bad), first, 8)
    assert rc == 0, lg.lib().lg_last_error(None)
    xs = [np.array([first[i]], np.uint32).view(np.float32)[0] for i in range(min(bad.value, 8))]
    return bad.value, xs


@pytest.mark.parametrize("fn,name", [(0, "exp"), (1, "log"), (2, "atan"), (3, "atanh"), (4, "sin"), (5, "cos"),
                                     (6, "pow(x, fixed y)"), (7, "atan2(x, p)"), (8, "pow(|x|, p)")])
def test_every_float_input(native, fn, name):
    bad, xs = sweep(fn)
    print(f"{name}: {bad} of 2^32 inputs differ from the double evaluation {xs}")
    assert bad == 0, xs


def test_probe_values(native):
    """The vector probe (fn 6-9) gives the same values as the sweep checks,
    on a few inputs the likelihood meets: Sersic arguments, SIE angles."""
    x = np.array([-0.5, 3.25, -87.2, -95.0, 1e-3, 0.7, 12.5, 1.0], np.float32)
    fp = C.POINTER(C.c_float)
    for fn, ref in ((6, np.exp), (7, np.log), (8, np.arctan), (9, np.arctanh)):
        xin = x if fn != 9 else np.clip(np.abs(x), 0, 0.99).astype(np.float32)
        if fn == 7:
            xin = np.abs(x) + np.float32(1e-3)
        out = np.empty_like(xin)
        rc = lg.lib().lg_probe_pair_math(0, fn, xin.ctypes.data_as(fp), xin.size, out.ctypes.data_as(fp))
        assert rc == 0
        want = ref(xin.astype(np.float64)).astype(np.float32)
        assert np.array_equal(out, want), (fn, out, want)
