"""lensed_gb300: GB300-native likelihood path of the strong-lensing code Lensed.

The product is the C-ABI library ``liblensed_gb300.so`` (declared in
``include/lensed_gb300.h``); this module is a thin ctypes binding to it for
Python callers and tests.  There is no Python or CPU fallback: if the library
is missing, importing the binding raises.

Typical use::

    import lensed_gb300 as lg
    ctx = lg.Context(image, weight, objects=[("lens", "sie_plus_shear", priors),
                                             ("src", "sersic", priors)],
                     psf=psf, rule="sub5", max_batch=1024)
    logL = ctx.eval_batch(params)        # (B, npars) physical values, map order
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

__all__ = ["Context", "Systems", "LensedError", "lib", "plugins", "plugin_params", "quad_rules", "make_weight",
           "compile_check", "write_fits", "fits_bytes", "DUMP_LAYERS", "LIB_PATH"]

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "liblensed_gb300.so")

LG_OK = 0
STATUS = {-1: "input", -2: "compile", -3: "cuda", -4: "alloc", -5: "timeout", -6: "unsupported"}
LG_FLAG_STRICT_FP = 1
LG_FLAG_NO_GRAPH = 2
LG_FLAG_IEEE_DIV = 4
LG_FLAG_AUTOTUNE = 8
LG_FLAG_FAST_MATH = 16
SHAPE_FIELDS = ("rt", "rppt", "qs", "ctx", "cty", "cr", "pair_rows")
DUMP_LAYERS = ("IMG", "RES", "RAW", "ERR", "WHT", "PVL")


class LensedError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{STATUS.get(code, code)}] {msg}")
        self.code = code


class _ImageDesc(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("image", C.POINTER(C.c_float)),
                ("weight", C.POINTER(C.c_float)), ("psf", C.POINTER(C.c_float)), ("psf_width", C.c_int),
                ("psf_height", C.c_int), ("pcs", C.c_double * 4)]


class _ObjectDesc(C.Structure):
    _fields_ = [("name", C.c_char_p), ("id", C.c_char_p), ("priors", C.POINTER(C.c_char_p))]


class NestedOptions(C.Structure):
    _fields_ = [("nlive", C.c_int), ("tol", C.c_double), ("efr", C.c_double), ("batch", C.c_int),
                ("seed", C.c_int), ("maxiter", C.c_long), ("proposal", C.c_int), ("flow_every", C.c_int),
                ("wrap", C.POINTER(C.c_int)), ("checkpoint", C.c_char_p), ("checkpoint_every", C.c_int),
                ("resume", C.c_int), ("max_ellipsoids", C.c_int), ("ceff", C.c_int)]


class NestedResult(C.Structure):
    _fields_ = [("logz", C.c_double), ("logz_err", C.c_double), ("information", C.c_double),
                ("max_logl", C.c_double), ("ncall", C.c_long), ("niter", C.c_long), ("nsamples", C.c_long),
                ("n_flow_proposals", C.c_long), ("n_ellipsoid_proposals", C.c_long), ("wall_s", C.c_double),
                ("mean", C.POINTER(C.c_double)), ("std", C.POINTER(C.c_double)),
                ("samples", C.POINTER(C.c_double)), ("sample_logwt", C.POINTER(C.c_double)),
                ("max_samples", C.c_long), ("eval_s", C.c_double), ("train_s", C.c_double),
                ("propose_s", C.c_double)]


class FlowOptions(C.Structure):
    _fields_ = [("layers", C.c_int), ("width", C.c_int), ("hidden", C.c_int), ("epochs", C.c_int),
                ("batch", C.c_int), ("lr", C.c_double), ("expand", C.c_double), ("patience", C.c_int),
                ("lag", C.c_int), ("draw_cost", C.c_double), ("wait_tries", C.c_int), ("train_tc", C.c_int)]


BATCH_LOGLIKE = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double))
PROPOSAL_ELLIPSOID, PROPOSAL_FLOW = 0, 1


class _Options(C.Structure):
    _fields_ = [("rule", C.c_char_p), ("device", C.c_int), ("max_batch", C.c_int), ("flags", C.c_int)]


_lib = None


def lib():
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(LIB_PATH)
    dp, fp, ip, vp = C.POINTER(C.c_double), C.POINTER(C.c_float), C.POINTER(C.c_int), C.c_void_p
    sig = {
        "lg_version": (C.c_char_p, []),
        "lg_plugin_count": (C.c_int, []),
        "lg_plugin_info": (C.c_int, [C.c_int, C.POINTER(C.c_char_p), ip, ip]),
        "lg_plugin_param": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_char_p), ip, fp, fp, fp]),
        "lg_quad_rule_count": (C.c_int, []),
        "lg_quad_rule_info": (C.c_int, [C.c_int, C.POINTER(C.c_char_p), ip, dp, dp, dp]),
        "lg_make_weight": (C.c_long, [fp, C.c_long, fp, fp, C.c_double, C.c_double, fp, ip, fp]),
        "lg_compile_check": (C.c_int, [C.POINTER(_ImageDesc), C.POINTER(_ObjectDesc), C.c_int,
                                       C.POINTER(_Options), C.c_char_p, C.c_size_t]),
        "lg_create": (vp, [C.POINTER(_ImageDesc), C.POINTER(_ObjectDesc), C.c_int, C.POINTER(_Options), ip]),
        "lg_destroy": (None, [vp]),
        "lg_last_error": (C.c_char_p, [vp]),
        "lg_npars": (C.c_int, [vp]),
        "lg_ndims": (C.c_int, [vp]),
        "lg_masked": (C.c_long, [vp]),
        "lg_pmap": (C.c_int, [vp, C.c_int]),
        "lg_param": (C.c_int, [vp, C.c_int, C.POINTER(C.c_char_p), ip, dp, dp]),
        "lg_eval_batch": (C.c_int, [vp, dp, C.c_int, dp]),
        "lg_eval_batch_device": (C.c_int, [vp, vp, C.c_int, vp, vp]),
        "lg_eval_cube_batch": (C.c_int, [vp, dp, C.c_int, dp, dp]),
        "lg_eval_cube_batch_device": (C.c_int, [vp, vp, C.c_int, vp, vp, vp]),
        "lg_render": (C.c_int, [vp, dp, fp, fp, fp]),
        "lg_dump": (C.c_int, [vp, dp, fp]),
        "lg_write_output": (C.c_int, [vp, dp, C.c_char_p]),
        "lg_write_fits": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.POINTER(fp), C.POINTER(C.c_char_p)]),
        "lg_write_fits_memory": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(fp), C.POINTER(C.c_char_p), vp,
                                           C.c_size_t, C.POINTER(C.c_size_t)]),
        "lg_eval_profile": (C.c_int, [vp, vp, C.c_int, vp, fp]),
        "lg_launch_shape": (C.c_int, [vp, ip]),
        "lg_set_launch_shape": (C.c_int, [vp, ip]),
        "lg_tune_report": (C.c_char_p, [vp]),
        "lg_host_set_active": (C.c_int, [vp]),
        "lg_tune_candidates": (C.c_int, [C.POINTER(_ImageDesc), C.POINTER(_ObjectDesc), C.c_int,
                                         C.POINTER(_Options), ip, C.c_int]),
        "lg_compile_check_shape": (C.c_int, [C.POINTER(_ImageDesc), C.POINTER(_ObjectDesc), C.c_int,
                                             C.POINTER(_Options), ip, C.c_char_p, C.c_size_t]),
        "lg_systems_launch_shape": (C.c_int, [vp, ip]),
        "lg_systems_set_launch_shape": (C.c_int, [vp, ip]),
        "lg_systems_tune_report": (C.c_char_p, [vp]),
        "lg_measure_fp32_peak": (C.c_int, [C.c_int, dp]),
        "lg_probe_pair_math": (C.c_int, [C.c_int, C.c_int, fp, C.c_int, fp]),
        "lg_probe_crf_sweep": (C.c_int, [C.c_int, C.c_int, C.c_ulonglong, C.c_ulonglong,
                                         C.POINTER(C.c_ulonglong), C.POINTER(C.c_uint), C.c_int]),
        "lg_loglike_images_noalloc": (C.c_int, [vp, vp, vp, C.c_long, C.c_int, vp, vp]),
        "lg_systems_create": (vp, [C.POINTER(_ImageDesc), C.c_int, C.POINTER(_ObjectDesc), C.c_int,
                                   C.POINTER(_Options), ip, ip]),
        "lg_systems_destroy": (None, [vp]),
        "lg_systems_last_error": (C.c_char_p, [vp]),
        "lg_systems_npars": (C.c_int, [vp]),
        "lg_systems_eval": (C.c_int, [vp, dp, ip, dp]),
        "lg_nested_defaults": (NestedOptions, []),
        "lg_flow_defaults": (FlowOptions, []),
        "lg_nested_sample": (C.c_int, [C.c_int, BATCH_LOGLIKE, vp, C.POINTER(NestedOptions),
                                       C.POINTER(NestedResult)]),
        "lg_nested_sample_flow": (C.c_int, [C.c_int, BATCH_LOGLIKE, vp, C.POINTER(NestedOptions),
                                            C.POINTER(FlowOptions), C.c_int, C.POINTER(NestedResult)]),
        "lg_nested_run": (C.c_int, [vp, C.POINTER(NestedOptions), C.POINTER(FlowOptions),
                                    C.POINTER(NestedResult)]),
        "lg_flow_nparams": (C.c_long, [C.c_int, C.c_int, C.c_int, C.c_int]),
        "lg_flow_inverse_check": (C.c_int, [C.c_int] * 7 + [fp, fp, C.c_int, fp, fp]),
        "lg_flow_inverse_time": (C.c_int, [C.c_int] * 6 + [fp, fp, C.c_int, C.c_int, fp]),
        "lg_flow_train_time": (C.c_int, [C.c_int] * 6 + [fp, fp, C.c_int, C.c_int, C.c_int, fp]),
        "lg_ellipsoid_draw_check": (C.c_int, [C.c_int, C.c_int, C.c_int, dp, dp, ip, dp, C.c_int, C.c_ulonglong]),
        "lg_flow_fit": (C.c_int, [C.c_int, C.c_int, C.POINTER(FlowOptions), dp, C.c_int, fp, C.c_int, dp]),
        "lg_flow_loss_grad": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, fp, fp, C.c_int,
                                        fp, fp]),
        "loglike": (None, [dp, ip, ip, dp, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _f32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float32)


def _p(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def plugins():
    """List of (name, kind, npars) of the registered object plugins."""
    L = lib()
    out = []
    for i in range(L.lg_plugin_count()):
        n, k, p = C.c_char_p(), C.c_int(), C.c_int()
        L.lg_plugin_info(i, C.byref(n), C.byref(k), C.byref(p))
        out.append((n.value.decode(), chr(k.value), p.value))
    return out


def plugin_params(name: str):
    """Parameters of a plugin: list of (name, type, lower, upper, default)."""
    L = lib()
    out = []
    j = 0
    while True:
        n, t, lo, hi, dv = C.c_char_p(), C.c_int(), C.c_float(), C.c_float(), C.c_float()
        if L.lg_plugin_param(name.encode(), j, C.byref(n), C.byref(t), C.byref(lo), C.byref(hi), C.byref(dv)):
            break
        out.append((n.value.decode(), t.value, lo.value, hi.value, dv.value))
        j += 1
    if not out:
        raise ValueError(f"unknown object: {name}")
    return out


def quad_rules():
    """Dict name -> (absc (n,2), weights (n,), errors (n,)) from the library."""
    L = lib()
    out = {}
    for i in range(L.lg_quad_rule_count()):
        n, s = C.c_char_p(), C.c_int()
        L.lg_quad_rule_info(i, C.byref(n), C.byref(s), None, None, None)
        a = np.zeros((s.value, 2)); w = np.zeros(s.value); e = np.zeros(s.value)
        L.lg_quad_rule_info(i, None, None, _p(a, C.c_double), _p(w, C.c_double), _p(e, C.c_double))
        out[n.value.decode()] = (a, w, e)
    return out


def measure_fp32_peak(device: int = 0) -> float:
    """Measured FP32 FMA throughput of the device in TFLOP/s."""
    v = C.c_double()
    rc = lib().lg_measure_fp32_peak(device, C.byref(v))
    if rc:
        raise LensedError(rc, "fp32 peak probe")
    return v.value


def _nested_opts(**kw):
    o = lib().lg_nested_defaults()
    for k, v in kw.items():
        if not hasattr(o, k):
            raise TypeError(f"unknown nested option {k}")
        if k == "checkpoint" and isinstance(v, str):
            v = os.fsencode(v)
        if k == "wrap":
            # periodic dimensions: a sequence of flags, kept alive with the options
            arr = (C.c_int * len(v))(*[int(bool(x)) for x in v])
            o._wrap_keep = arr
            v = C.cast(arr, C.POINTER(C.c_int))
        setattr(o, k, v)
    return o


def _flow_opts(**kw):
    o = lib().lg_flow_defaults()
    for k, v in kw.items():
        if not hasattr(o, k):
            raise TypeError(f"unknown flow option {k}")
        setattr(o, k, v)
    return o


def _result(nd, max_samples):
    r = NestedResult()
    arrays = {"mean": np.zeros(nd), "std": np.zeros(nd), "samples": np.zeros((max_samples, nd)),
              "logwt": np.zeros(max_samples)}
    r.mean, r.std = _p(arrays["mean"], C.c_double), _p(arrays["std"], C.c_double)
    r.samples, r.sample_logwt = _p(arrays["samples"], C.c_double), _p(arrays["logwt"], C.c_double)
    r.max_samples = max_samples
    return r, arrays


def _pack(r, arrays):
    n = min(r.nsamples, r.max_samples)
    return {"logz": r.logz, "logz_err": r.logz_err, "information": r.information, "max_logl": r.max_logl,
            "ncall": r.ncall, "niter": r.niter, "nsamples": r.nsamples, "wall_s": r.wall_s,
            "eval_s": r.eval_s, "train_s": r.train_s, "propose_s": r.propose_s,
            "n_flow_proposals": r.n_flow_proposals, "n_ellipsoid_proposals": r.n_ellipsoid_proposals,
            "mean": arrays["mean"], "std": arrays["std"], "samples": arrays["samples"][:n],
            "logwt": arrays["logwt"][:n]}


def flow_fit(points, device: int = 0, **flow):
    """One retraining of the learned proposal on points (n, d), as the
    sampler retrains on its live points: returns (held-out loss before
    training and after each epoch, calibrated kept fraction)."""
    x = np.ascontiguousarray(points, dtype=np.float64)
    hist = np.full(256, np.nan, np.float32)
    eff = C.c_double()
    fo = _flow_opts(**flow)
    rc = lib().lg_flow_fit(device, x.shape[1], C.byref(fo), _p(x, C.c_double), x.shape[0], _p(hist, C.c_float),
                           hist.size, C.byref(eff))
    if rc < 0:
        raise LensedError(rc, lib().lg_last_error(None).decode(errors="replace"))
    return hist[: rc + 1], eff.value


def nested_sample(loglike, ndims: int, max_samples: int = 200000, **opts):
    """Nested sampling of a batched log-likelihood over the unit cube.

    loglike(cube) receives a (B, ndims) array and returns B log-likelihoods."""
    err = []

    def cb(_user, cube, B, out):
        try:
            x = np.ctypeslib.as_array(cube, shape=(B, ndims))
            res = np.asarray(loglike(x.copy()), dtype=np.float64)
            np.ctypeslib.as_array(out, shape=(B,))[:] = res
            return 0
        except Exception as e:  # reported after the call
            err.append(e)
            return -1

    f = BATCH_LOGLIKE(cb)
    o = _nested_opts(**opts)
    r, arrays = _result(ndims, max_samples)
    rc = lib().lg_nested_sample(ndims, f, None, C.byref(o), C.byref(r))
    if err:
        raise err[0]
    if rc:
        raise LensedError(rc, lib().lg_last_error(None).decode(errors="replace"))
    return _pack(r, arrays)


def nested_sample_flow(loglike, ndims: int, max_samples: int = 200000, flow: dict | None = None, device: int = 0,
                       **opts):
    """nested_sample with the learned coupling-flow proposal (needs a GPU)."""
    err = []

    def cb(_user, cube, B, out):
        try:
            x = np.ctypeslib.as_array(cube, shape=(B, ndims))
            np.ctypeslib.as_array(out, shape=(B,))[:] = np.asarray(loglike(x.copy()), dtype=np.float64)
            return 0
        except Exception as e:
            err.append(e)
            return -1

    f = BATCH_LOGLIKE(cb)
    o = _nested_opts(**opts)
    o.proposal = PROPOSAL_FLOW
    fo = _flow_opts(**(flow or {}))
    r, arrays = _result(ndims, max_samples)
    rc = lib().lg_nested_sample_flow(ndims, f, None, C.byref(o), C.byref(fo), device, C.byref(r))
    if err:
        raise err[0]
    if rc:
        raise LensedError(rc, lib().lg_last_error(None).decode(errors="replace"))
    return _pack(r, arrays)


def _layer_args(layers, names):
    arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in layers]
    if not arrs or any(a.ndim != 2 or a.shape != arrs[0].shape for a in arrs):
        raise ValueError("layers must be 2-D arrays of one shape")
    ptrs = (C.POINTER(C.c_float) * len(arrs))(*[_p(a, C.c_float) for a in arrs])
    nm = None
    if names is not None:
        if len(names) != len(arrs):
            raise ValueError("one name per layer")
        nm = (C.c_char_p * len(arrs))(*[None if n is None else n.encode() for n in names])
    H, W = arrs[0].shape
    return arrs, ptrs, nm, W, H


def _global_check(rc):
    if rc != LG_OK:
        raise LensedError(rc, lib().lg_last_error(None).decode())


def write_fits(path: str, layers, names=None) -> None:
    """Write 2-D float32 layers as IMAGE extensions of a FITS file (after an
    empty primary HDU), named by EXTNAME when names are given."""
    arrs, ptrs, nm, W, H = _layer_args(layers, names)
    _global_check(lib().lg_write_fits(os.fsencode(path), W, H, len(arrs), ptrs, nm))


def fits_bytes(layers, names=None) -> bytes:
    """The FITS file write_fits would write, as bytes."""
    arrs, ptrs, nm, W, H = _layer_args(layers, names)
    size = C.c_size_t()
    _global_check(lib().lg_write_fits_memory(W, H, len(arrs), ptrs, nm, None, 0, C.byref(size)))
    buf = C.create_string_buffer(size.value)
    _global_check(lib().lg_write_fits_memory(W, H, len(arrs), ptrs, nm, buf, size.value, C.byref(size)))
    return buf.raw[: size.value]


def make_weight(image, weight_map=None, gain=None, gain_value=1.0, offset=0.0, xweight=None, mask=None):
    """Weights as Lensed builds them; returns (weight, masked_count)."""
    img = _f32(image)
    out = np.zeros_like(img)
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.int32)
    wm, g, xw = _f32(weight_map), _f32(gain), _f32(xweight)
    n = lib().lg_make_weight(_p(img, C.c_float), img.size, _p(wm, C.c_float), _p(g, C.c_float), float(gain_value),
                             float(offset), _p(xw, C.c_float), _p(m, C.c_int), _p(out, C.c_float))
    if n < 0:
        raise LensedError(int(n), "make_weight")
    return out, int(n)


def _objects(objects):
    """objects: sequence of plugin names, (id, name) or (id, name, priors)."""
    keep = []
    arr = (_ObjectDesc * len(objects))()
    for i, o in enumerate(objects):
        if isinstance(o, str):
            oid, name, pri = None, o, None
        elif len(o) == 2:
            (oid, name), pri = o, None
        else:
            oid, name, pri = o
        arr[i].name = name.encode()
        arr[i].id = oid.encode() if oid else None
        if pri is not None:
            if isinstance(pri, dict):
                pnames = [p[0] for p in plugin_params(name)]
                pri = [pri.get(pn) for pn in pnames]
            pa = (C.c_char_p * len(pri))(*[(None if v is None else str(v).encode()) for v in pri])
            keep.append(pa)
            arr[i].priors = C.cast(pa, C.POINTER(C.c_char_p))
    return arr, keep


def _image_desc(width, height, image, weight, psf, pcs):
    d = _ImageDesc()
    d.width, d.height = int(width), int(height)
    d.image = _p(image, C.c_float)
    d.weight = _p(weight, C.c_float)
    if psf is not None:
        d.psf = _p(psf, C.c_float)
        d.psf_height, d.psf_width = psf.shape
    if pcs is not None:
        for i in range(4):
            d.pcs[i] = float(pcs[i])
    return d


def _options(rule, device, max_batch, flags):
    o = _Options()
    o.rule = rule.encode() if rule else None
    o.device, o.max_batch, o.flags = int(device), int(max_batch), int(flags)
    return o


def compile_check(width, height, objects, psf=None, rule="g3k7", pcs=None, flags=0):
    """Compose and compile a model with NVRTC without a GPU; returns the log."""
    psf_a = _f32(psf)
    arr, keep = _objects(objects)
    d = _image_desc(width, height, None, None, psf_a, pcs)
    buf = C.create_string_buffer(1 << 16)
    rc = lib().lg_compile_check(C.byref(d), arr, len(objects), C.byref(_options(rule, 0, 0, flags)), buf, len(buf))
    if rc:
        raise LensedError(rc, buf.value.decode(errors="replace"))
    return buf.value.decode(errors="replace")


def tune_candidates(width, height, objects, psf=None, rule="g3k7", pcs=None, flags=0):
    """The launch shapes the autotuner times for a model (list of dicts)."""
    psf_a = _f32(psf)
    arr, keep = _objects(objects)
    d = _image_desc(width, height, None, None, psf_a, pcs)
    buf = (C.c_int * (7 * 64))()
    n = lib().lg_tune_candidates(C.byref(d), arr, len(objects), C.byref(_options(rule, 0, 0, flags)), buf, 64)
    if n < 0:
        raise LensedError(n, lib().lg_last_error(None).decode(errors="replace"))
    return [dict(zip(SHAPE_FIELDS, list(buf[7 * i: 7 * i + 7]))) for i in range(min(n, 64))]


def compile_check_shape(width, height, objects, shape: dict, psf=None, rule="g3k7", pcs=None, flags=0):
    """compile_check of the evaluation module for one launch shape."""
    psf_a = _f32(psf)
    arr, keep = _objects(objects)
    d = _image_desc(width, height, None, None, psf_a, pcs)
    v = (C.c_int * 7)(*[int(shape[k]) for k in SHAPE_FIELDS])
    buf = C.create_string_buffer(1 << 16)
    rc = lib().lg_compile_check_shape(C.byref(d), arr, len(objects), C.byref(_options(rule, 0, 0, flags)), v, buf,
                                      len(buf))
    if rc:
        raise LensedError(rc, buf.value.decode(errors="replace"))
    return buf.value.decode(errors="replace")


class Systems:
    """A batch of lens systems sharing the objects (wraps lg_systems_*).

    systems: sequence of (image, weight, psf-or-None, pcs-or-None);
    capacity: max candidates per system per call."""

    def __init__(self, systems, objects: Sequence, capacity, rule: str = "g3k7", device: int = 0,
                 flags: int = 0):
        L = lib()
        self._keep = []
        descs = (_ImageDesc * len(systems))()
        for i, (img, wht, psf, pcs) in enumerate(systems):
            a, w = _f32(img), _f32(wht)
            p = _f32(psf)
            self._keep += [a, w, p]
            descs[i] = _image_desc(a.shape[1], a.shape[0], a, w, p, pcs)
        arr, keep = _objects(objects)
        self._keep += [arr, keep]
        cap = np.ascontiguousarray(capacity, dtype=np.int32)
        self.capacity = cap
        st = C.c_int()
        self.h = L.lg_systems_create(descs, len(systems), arr, len(objects),
                                     C.byref(_options(rule, device, 0, flags)), _p(cap, C.c_int), C.byref(st))
        if not self.h:
            raise LensedError(st.value, L.lg_last_error(None).decode(errors="replace"))
        self.nsys = len(systems)
        self.npars = L.lg_systems_npars(self.h)

    def close(self):
        if getattr(self, "h", None):
            lib().lg_systems_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    @property
    def launch_shape(self) -> dict:
        """Launch shape of the multi-system kernels (see lg_systems_launch_shape)."""
        v = (C.c_int * 7)()
        lib().lg_systems_launch_shape(self.h, v)
        return dict(zip(SHAPE_FIELDS, list(v)))

    def set_launch_shape(self, **shape) -> None:
        """Recompile the kernels for a launch shape (fields of SHAPE_FIELDS;
        missing ones keep their current value)."""
        cur = self.launch_shape
        cur.update(shape)
        v = (C.c_int * 7)(*[int(cur[k]) for k in SHAPE_FIELDS])
        rc = lib().lg_systems_set_launch_shape(self.h, v)
        if rc:
            raise LensedError(rc, lib().lg_systems_last_error(self.h).decode(errors="replace"))

    @property
    def tune_report(self) -> str:
        return lib().lg_systems_tune_report(self.h).decode()

    def eval(self, params_list):
        """params_list: per system a (count, npars) array in map order."""
        counts = np.array([len(p) for p in params_list], dtype=np.int32)
        flat = np.ascontiguousarray(np.concatenate([np.asarray(p, np.float64).reshape(-1, self.npars)
                                                    for p in params_list]))
        out = np.empty(int(counts.sum()))
        rc = lib().lg_systems_eval(self.h, _p(flat, C.c_double), _p(counts, C.c_int), _p(out, C.c_double))
        if rc:
            raise LensedError(rc, lib().lg_systems_last_error(self.h).decode(errors="replace"))
        return np.split(out, np.cumsum(counts)[:-1])


class Context:
    """One lens system resident on a GPU (wraps lg_create/lg_eval_batch)."""

    def __init__(self, image, weight, objects: Sequence, psf=None, rule: str = "g3k7", pcs=None,
                 device: int = 0, max_batch: int = 1024, flags: int = 0):
        L = lib()
        self._image = _f32(image)
        self._weight = _f32(weight)
        self._psf = _f32(psf)
        h, w = self._image.shape
        arr, keep = _objects(objects)
        d = _image_desc(w, h, self._image, self._weight, self._psf, pcs)
        st = C.c_int()
        self.h = L.lg_create(C.byref(d), arr, len(objects), C.byref(_options(rule, device, max_batch, flags)),
                             C.byref(st))
        if not self.h:
            raise LensedError(st.value, L.lg_last_error(None).decode(errors="replace"))
        self.width, self.height = w, h
        self.npars = L.lg_npars(self.h)
        self.ndims = L.lg_ndims(self.h)
        self.max_batch = max_batch
        self.pmap = [L.lg_pmap(self.h, i) for i in range(self.npars)]
        self.ids = []
        for i in range(self.npars):
            s = C.c_char_p()
            L.lg_param(self.h, i, C.byref(s), None, None, None)
            self.ids.append(s.value.decode())

    def close(self):
        if getattr(self, "h", None):
            lib().lg_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc):
        if rc:
            raise LensedError(rc, lib().lg_last_error(self.h).decode(errors="replace"))

    @property
    def masked(self) -> int:
        return lib().lg_masked(self.h)

    @property
    def launch_shape(self) -> dict:
        """Launch shape of the evaluation kernels (see lg_launch_shape)."""
        v = (C.c_int * 7)()
        self._check(lib().lg_launch_shape(self.h, v))
        return dict(zip(SHAPE_FIELDS, list(v)))

    def set_launch_shape(self, **shape) -> None:
        """Recompile the evaluation kernels for a launch shape (fields of
        SHAPE_FIELDS; missing ones keep their current value)."""
        cur = self.launch_shape
        cur.update(shape)
        v = (C.c_int * 7)(*[int(cur[k]) for k in SHAPE_FIELDS])
        self._check(lib().lg_set_launch_shape(self.h, v))

    @property
    def tune_report(self) -> str:
        """The autotuner's candidates and timings ("" if not tuned)."""
        return lib().lg_tune_report(self.h).decode()

    @property
    def host_set(self) -> bool:
        """Batches of up to 4 candidates take their object data from the host."""
        return bool(lib().lg_host_set_active(self.h))

    def to_map_order(self, params_obj):
        """Reorder (..., npars) parameters from object order to map order
        (C-contiguous, ready for the device entry points)."""
        p = np.asarray(params_obj, dtype=np.float64)
        return np.ascontiguousarray(p[..., self.pmap])

    def eval_batch(self, params) -> np.ndarray:
        p = np.ascontiguousarray(np.atleast_2d(params), dtype=np.float64)
        if p.shape[1] != self.npars:
            raise ValueError(f"expected {self.npars} parameters, got {p.shape[1]}")
        out = np.empty(p.shape[0])
        for b0 in range(0, p.shape[0], self.max_batch):
            blk = np.ascontiguousarray(p[b0:b0 + self.max_batch])
            self._check(lib().lg_eval_batch(self.h, _p(blk, C.c_double), blk.shape[0],
                                            out[b0:b0 + blk.shape[0]].ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def eval_batch_device(self, d_params: int, B: int, d_logL: int, stream: int = 0) -> None:
        """Device-pointer variant (e.g. torch tensors' data_ptr()); asynchronous."""
        self._check(lib().lg_eval_batch_device(self.h, C.c_void_p(d_params), int(B), C.c_void_p(d_logL),
                                               C.c_void_p(stream) if stream else None))

    def profile(self, d_params: int, B: int, d_logL: int):
        """Device ms of (set_params, render, convolve, finish) for one evaluation."""
        ms = np.zeros(4, np.float32)
        self._check(lib().lg_eval_profile(self.h, C.c_void_p(d_params), int(B), C.c_void_p(d_logL),
                                          _p(ms, C.c_float)))
        return ms

    def eval_cube(self, cube):
        u = np.ascontiguousarray(np.atleast_2d(cube), dtype=np.float64)
        phys = np.empty((u.shape[0], self.npars))
        out = np.empty(u.shape[0])
        self._check(lib().lg_eval_cube_batch(self.h, _p(u, C.c_double), u.shape[0], _p(phys, C.c_double),
                                             _p(out, C.c_double)))
        return out, phys

    def eval_cube_device(self, d_cube: int, B: int, d_phys: int, d_logL: int, stream: int = 0) -> None:
        """Unit-cube evaluation with device pointers (prior transform on the
        GPU); d_phys may be 0; asynchronous on the given stream."""
        self._check(lib().lg_eval_cube_batch_device(self.h, C.c_void_p(d_cube or None), int(B),
                                                    C.c_void_p(d_phys or None), C.c_void_p(d_logL),
                                                    C.c_void_p(stream) if stream else None))

    def render(self, params):
        """(model, raw, error) images for one parameter vector (map order)."""
        p = np.ascontiguousarray(params, dtype=np.float64)
        shp = (self.height, self.width)
        m, r, e = np.empty(shp, np.float32), np.empty(shp, np.float32), np.empty(shp, np.float32)
        self._check(lib().lg_render(self.h, _p(p, C.c_double), _p(m, C.c_float), _p(r, C.c_float),
                                    _p(e, C.c_float)))
        return m, r, e

    def dump(self, params):
        """The dumper's output layers for one parameter vector (map order):
        a dict IMG, RES, RAW, ERR, WHT, PVL -> (H, W) float32 array."""
        p = np.ascontiguousarray(params, dtype=np.float64)
        out = np.empty((len(DUMP_LAYERS), self.height, self.width), np.float32)
        self._check(lib().lg_dump(self.h, _p(p, C.c_double), _p(out, C.c_float)))
        return {n: out[i] for i, n in enumerate(DUMP_LAYERS)}

    def write_output(self, params, path: str) -> None:
        """Write the dumper's layers for one parameter vector to a FITS file."""
        p = np.ascontiguousarray(params, dtype=np.float64)
        self._check(lib().lg_write_output(self.h, _p(p, C.c_double), os.fsencode(path)))

    def nested(self, max_samples: int = 200000, flow: dict | None = None, **opts):
        """Nested sampling of this context's posterior (unit-cube means/samples)."""
        o = _nested_opts(**opts)
        fo = _flow_opts(**(flow or {}))
        r, arrays = _result(self.ndims, max_samples)
        self._check(lib().lg_nested_run(self.h, C.byref(o), C.byref(fo), C.byref(r)))
        return _pack(r, arrays)

    def loglike(self, cube):
        """The reference callback signature: returns (logL, physical params)."""
        c = np.zeros(self.npars)
        c[: self.ndims] = cube
        nd, npar, lnew = C.c_int(self.ndims), C.c_int(self.npars), C.c_double()
        lib().loglike(_p(c, C.c_double), C.byref(nd), C.byref(npar), C.byref(lnew), C.c_void_p(self.h))
        return lnew.value, c
