"""The allocation-free chi^2 entry point, checked against lg_eval_batch.

lg_loglike_images_noalloc serves callers that cannot allocate device memory
(a framework that owns the GPU's memory, or code where allocation is not
allowed): it reduces model images the caller already holds, with its scratch
in a static device array.  Its logL must agree with the context's own
evaluation of the same parameters (whose model images come from lg_render)
to within the strict-mode logL tolerance, on two calls in a row (the second
call reuses the scratch left by the first).  The first call in a process may
load the library's kernels and place the static array (CUDA's lazy module
loading); the second must leave the device's free memory unchanged.
"""
import ctypes as C

import numpy as np
import pytest

import lensed_gb300 as lg
from lensed_gb300 import workloads

pytestmark = pytest.mark.gpu


def _dev(a, torch):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_noalloc_loglike_matches_eval_batch_twice(native):
    torch = pytest.importorskip("torch")
    s = workloads.config2()
    B = 6
    ctx = lg.Context(s.image, s.weight, s.objects, psf=s.psf, rule=s.rule, max_batch=B)
    params = ctx.to_map_order(workloads.draw_candidates(s, B, seed=11))
    want = ctx.eval_batch(params)
    models = np.stack([ctx.render(p)[0] for p in params]).astype(np.float32)
    d_img, d_w = _dev(s.image, torch), _dev(s.weight, torch)
    d_models = _dev(models, torch)
    N = s.width * s.height
    # every output buffer exists before the first call
    outs = [torch.full((B,), np.nan, dtype=torch.float64, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    free = []
    for call in range(2):
        free.append(torch.cuda.mem_get_info()[0])
        rc = lg.lib().lg_loglike_images_noalloc(C.c_void_p(d_img.data_ptr()), C.c_void_p(d_w.data_ptr()),
                                                C.c_void_p(d_models.data_ptr()), N, B,
                                                C.c_void_p(outs[call].data_ptr()), None)
        assert rc == 0, lg.lib().lg_last_error(None)
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        got = outs[call].cpu().numpy()
        assert np.all(np.abs(got - want) <= 1e-6), (call, got - want)
    # the second call allocated nothing on the device
    assert free[3] == free[2], free


def test_noalloc_rejects_oversize_and_null(native):
    torch = pytest.importorskip("torch")
    d = torch.zeros(16, dtype=torch.float32, device="cuda")
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    p = C.c_void_p(d.data_ptr())
    rc = lg.lib().lg_loglike_images_noalloc(p, p, p, 16, 70000, C.c_void_p(out.data_ptr()), None)
    assert rc == -1 and b"maximum" in lg.lib().lg_last_error(None)
    rc = lg.lib().lg_loglike_images_noalloc(None, p, p, 16, 1, C.c_void_p(out.data_ptr()), None)
    assert rc == -1
