"""ctypes wrapper of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Imported by tests/, by ``__graft_entry__.smoke()`` and by the CPU-baseline
leg of bench.py, never by the product.  Builds ``oracle/liblensed_oracle.so``
from ``oracle/lensed_oracle.cpp`` on first use if it is missing.

``Oracle(objects, ...)`` models one lens system:
  objects   list of plugin names in list order ("sie", "sersic", "sky", ...)
            or (name, ipp) pairs where ipp marks an image-plane (x, y) prior
  width, height, pcs, rule (QuadRule), psf (2-D array or None),
  image / weight (2-D arrays, needed for logL)
  precision 32 (FP32 oracle) or 64 (FP64 oracle)
  math      FP32 per-ray elementary functions: "cr" (evaluated in double and
            rounded once: the strict semantics, the default) or "libm" (the C
            library's float functions).  set_params always uses "cr".
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liblensed_oracle.so")
SRC = os.path.join(HERE, "lensed_oracle.cpp")

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle: g++ -O2, no FMA contraction, OpenMP."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
               "-o", LIB, SRC]
        subprocess.check_call(cmd)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        dp = C.POINTER(C.c_double)
        fp = C.POINTER(C.c_float)
        ip = C.POINTER(C.c_int)
        L.lo_plugin_index.argtypes = [C.c_char_p]
        L.lo_plugin_npars.argtypes = [C.c_int]
        L.lo_plugin_kind.argtypes = [C.c_int]
        L.lo_create.restype = C.c_void_p
        L.lo_create.argtypes = [C.c_int, C.c_int, ip, ip, C.c_int, C.c_int, dp, C.c_int, dp, dp, dp, dp, fp,
                                C.c_int, C.c_int, fp, fp, C.c_int]
        L.lo_destroy.argtypes = [C.c_void_p]
        L.lo_npars.argtypes = [C.c_void_p]
        L.lo_set_threads.argtypes = [C.c_void_p, C.c_int]
        L.lo_render.argtypes = [C.c_void_p, dp, dp, dp, dp]
        L.lo_loglike_batch.argtypes = [C.c_void_p, dp, C.c_int, dp]
        L.lo_set_eval_cr.argtypes = [C.c_int]
        L.lo_make_weight.argtypes = [fp, C.c_long, fp, fp, C.c_double, C.c_double, fp, ip, fp]
        _lib = L
    return _lib


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


def plugin_npars(name: str) -> int:
    L = lib()
    i = L.lo_plugin_index(name.encode())
    if i < 0:
        raise ValueError(f"unknown object: {name}")
    return L.lo_plugin_npars(i)


class Oracle:
    def __init__(self, objects: Sequence, width: int, height: int, rule, pcs=(1.0, 1.0, 1.0, 1.0),
                 psf: Optional[np.ndarray] = None, image: Optional[np.ndarray] = None,
                 weight: Optional[np.ndarray] = None, precision: int = 32, threads: int = 1,
                 math: str = "cr"):
        if math not in ("cr", "libm"):
            raise ValueError("math must be 'cr' or 'libm'")
        self.math = math
        L = lib()
        names, ipps = [], []
        for o in objects:
            if isinstance(o, (tuple, list)):
                names.append(o[0]); ipps.append(int(bool(o[1])))
            else:
                names.append(o); ipps.append(0)
        ids = np.array([L.lo_plugin_index(n.encode()) for n in names], dtype=np.int32)
        if (ids < 0).any():
            raise ValueError(f"unknown object in {names}")
        ipp = np.array(ipps, dtype=np.int32)
        self.width, self.height = int(width), int(height)
        self.N = self.width * self.height
        pcs_a = np.array(pcs, dtype=np.float64)
        pts = np.array(rule.points, dtype=np.float64).reshape(-1, 2)
        qx, qy = np.ascontiguousarray(pts[:, 0]), np.ascontiguousarray(pts[:, 1])
        qw = np.array(rule.weights, dtype=np.float64)
        qe = np.array(rule.errors, dtype=np.float64)
        self._keep = [ids, ipp, pcs_a, qx, qy, qw, qe]
        psf_a = None if psf is None else np.ascontiguousarray(psf, dtype=np.float32)
        pw = ph = 0
        if psf_a is not None:
            ph, pw = psf_a.shape
        img = None if image is None else np.ascontiguousarray(image, dtype=np.float32).ravel()
        wht = None if weight is None else np.ascontiguousarray(weight, dtype=np.float32).ravel()
        self.has_psf = psf_a is not None
        self.precision = precision
        self.h = L.lo_create(precision, len(ids), _ptr(ids, C.c_int), _ptr(ipp, C.c_int), self.width, self.height,
                             _ptr(pcs_a, C.c_double), len(qw), _ptr(qx, C.c_double), _ptr(qy, C.c_double),
                             _ptr(qw, C.c_double), _ptr(qe, C.c_double), _ptr(psf_a, C.c_float), pw, ph,
                             _ptr(img, C.c_float), _ptr(wht, C.c_float), threads)
        if not self.h:
            raise ValueError("oracle: invalid model")
        self.npars = L.lo_npars(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().lo_destroy(self.h)
            self.h = None

    def set_threads(self, n: int) -> None:
        lib().lo_set_threads(self.h, n)

    def render(self, params):
        """Return (value, error, convolved-or-None) as (H, W) float64 arrays."""
        p = np.ascontiguousarray(params, dtype=np.float64)
        assert p.size == self.npars
        lib().lo_set_eval_cr(1 if self.math == "cr" else 0)
        v = np.zeros(self.N); e = np.zeros(self.N)
        c = np.zeros(self.N) if self.has_psf else None
        lib().lo_render(self.h, _ptr(p, C.c_double), _ptr(v, C.c_double), _ptr(e, C.c_double), _ptr(c, C.c_double))
        shp = (self.height, self.width)
        return v.reshape(shp), e.reshape(shp), (c.reshape(shp) if c is not None else None)

    def loglike(self, params):
        """logL for a (B, npars) array of parameter vectors in object order."""
        p = np.ascontiguousarray(np.atleast_2d(params), dtype=np.float64)
        assert p.shape[1] == self.npars
        out = np.zeros(p.shape[0])
        lib().lo_set_eval_cr(1 if self.math == "cr" else 0)
        rc = lib().lo_loglike_batch(self.h, _ptr(p, C.c_double), p.shape[0], _ptr(out, C.c_double))
        if rc:
            raise ValueError("oracle: image and weight are needed for logL")
        return out


DUMP_NAMES = ("IMG", "RES", "RAW", "ERR", "WHT", "PVL")


def dump_layers(image, weight, model, raw, error):
    """Oracle restatement of the dumper's output layers (src/nested.c:217-254)
    from a rendered model: IMG model, RES image - model, RAW unconvolved
    model, ERR error / RAW, WHT weight, PVL erfc(sqrt(chi2 / 2)) with the
    per-pixel chi2 = weight * (model - image)^2 of the loglike kernel
    (kernel/lensed.cl:41-53).  FP32 arithmetic as the reference's; the
    p-value in double (math.erfc per pixel), rounded to float32."""
    import math

    f = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    img, w, m, v, e = f(image), f(weight), f(model), f(raw), f(error)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = m - img
        chi2 = (w * r) * r
        relerr = e / v
    pvl = np.array([math.erfc(math.sqrt(0.5 * float(c))) for c in chi2.ravel()], dtype=np.float64)
    pvl = pvl.astype(np.float32).reshape(m.shape)
    return {"IMG": m, "RES": img - m, "RAW": v, "ERR": relerr, "WHT": w, "PVL": pvl}


def make_weight(image, weight_map=None, gain=None, gain_value=1.0, offset=0.0, xweight=None, mask=None):
    """Oracle restatement of Lensed's weight construction (float32 array)."""
    img = np.ascontiguousarray(image, dtype=np.float32).ravel()
    out = np.zeros_like(img)
    def f(a):
        return None if a is None else np.ascontiguousarray(a, dtype=np.float32).ravel()
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.int32).ravel()
    wm, g, xw = f(weight_map), f(gain), f(xweight)
    lib().lo_make_weight(_ptr(img, C.c_float), img.size, _ptr(wm, C.c_float), _ptr(g, C.c_float), float(gain_value),
                         float(offset), _ptr(xw, C.c_float), _ptr(m, C.c_int), _ptr(out, C.c_float))
    return out.reshape(np.shape(image))
