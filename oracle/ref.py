"""ctypes wrapper of the reference-built checker (oracle/_ref) -- TEST
INFRASTRUCTURE ONLY.  See oracle/build_ref.py for how it is built.

``Reference.for_model(objects, width, height, rule, psf, ...)`` loads the
library of that configuration; ``math`` selects the double-evaluated ("cr")
or the C library's ("libm") float functions.
"""
from __future__ import annotations

import ctypes as C
import os
import sys
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")

from oracle import build_ref  # noqa: E402


def _ptr(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def library_path(objects, width, height, psf_shape, nq, math="cr") -> str:
    name = build_ref.config_name([(o, int(i)) for o, i in objects], width, height, tuple(psf_shape), nq)
    return os.path.join(OUT, f"{name}_{math}.so")


def available(objects=None, width=None, height=None, psf_shape=(0, 0), nq=None, math="cr") -> bool:
    if objects is None:
        return os.path.isdir(OUT) and any(f.endswith(".so") and f.startswith("cfg_") for f in os.listdir(OUT))
    return os.path.exists(library_path(objects, width, height, psf_shape, nq, math))


class Reference:
    """One configuration of the reference's own likelihood code."""

    def __init__(self, objects: Sequence, width: int, height: int, rule, psf: Optional[np.ndarray] = None,
                 image: Optional[np.ndarray] = None, weight: Optional[np.ndarray] = None,
                 pcs=(1.0, 1.0, 1.0, 1.0), math: str = "cr", threads: int = 1):
        objs = [(o, 0) if isinstance(o, str) else (o[0], int(o[1])) for o in objects]
        psf_shape = (0, 0) if psf is None else (psf.shape[1], psf.shape[0])
        path = library_path(objs, width, height, psf_shape, rule.size, math)
        if not os.path.exists(path):
            raise FileNotFoundError(f"reference configuration not built: {path}")
        L = C.CDLL(path)
        dp, fp = C.POINTER(C.c_double), C.POINTER(C.c_float)
        L.ref_create.restype = C.c_void_p
        L.ref_create.argtypes = [fp, fp, fp, dp, C.c_int, dp, dp, dp, dp, C.c_int]
        L.ref_eval.restype = C.c_double
        L.ref_eval.argtypes = [C.c_void_p, fp, fp, fp, fp]
        L.ref_destroy.argtypes = [C.c_void_p]
        self.L = L
        self.npars = L.ref_npars()
        self.width, self.height, self.N = width, height, width * height
        pts = np.array(rule.points, np.float64).reshape(-1, 2)
        self._keep = [np.ascontiguousarray(pts[:, 0]), np.ascontiguousarray(pts[:, 1]),
                      np.array(rule.weights, np.float64), np.array(rule.errors, np.float64),
                      np.array(pcs, np.float64)]
        img = None if image is None else np.ascontiguousarray(image, np.float32).ravel()
        wht = None if weight is None else np.ascontiguousarray(weight, np.float32).ravel()
        ps = None if psf is None else np.ascontiguousarray(psf, np.float32)
        qx, qy, qw, qe, pc = self._keep
        self.h = L.ref_create(_ptr(img, C.c_float), _ptr(wht, C.c_float), _ptr(ps, C.c_float), _ptr(pc, C.c_double),
                              rule.size, _ptr(qx, C.c_double), _ptr(qy, C.c_double), _ptr(qw, C.c_double),
                              _ptr(qe, C.c_double), threads)
        if not self.h:
            raise ValueError("reference: invalid configuration")
        self.has_psf = psf is not None

    @classmethod
    def for_system(cls, s, threads: int = 1, math: str = "libm"):
        from lensed_gb300 import quadrature

        return cls(s.plugins, s.width, s.height, quadrature.rule(s.rule), psf=s.psf, image=s.image,
                   weight=s.weight, math=math, threads=threads)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_destroy(self.h)
            self.h = None

    def render(self, params):
        """(value, error, convolved-or-None) as (H, W) float32 arrays."""
        p = np.ascontiguousarray(np.asarray(params, np.float64).astype(np.float32))
        v = np.zeros(self.N, np.float32); e = np.zeros(self.N, np.float32)
        c = np.zeros(self.N, np.float32) if self.has_psf else None
        self.L.ref_eval(self.h, _ptr(p, C.c_float), _ptr(v, C.c_float), _ptr(e, C.c_float), _ptr(c, C.c_float))
        shp = (self.height, self.width)
        return v.reshape(shp), e.reshape(shp), (c.reshape(shp) if c is not None else None)

    def loglike(self, params):
        """logL of (B, npars) parameter vectors in object order."""
        p = np.atleast_2d(np.asarray(params, np.float64))
        out = np.zeros(p.shape[0])
        for b in range(p.shape[0]):
            pf = np.ascontiguousarray(p[b].astype(np.float32))
            out[b] = self.L.ref_eval(self.h, _ptr(pf, C.c_float), None, None, None)
        return out
