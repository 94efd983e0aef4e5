"""Oracle (test infrastructure): Lensed's parameter space and the unit-cube
prior transform, restated in numpy for checking the GPU transform.

Follows:
* prior definitions (src/prior.c, src/prior/{delta,unif,norm}.c): a bare
  number is a delta (pseudo) prior; ``unif a b``; ``norm mean sigma``, drawn
  through the inverse normal CDF of Abramowitz & Stegun 26.2.23
  (src/prior/norm.c:9-16) with support mean +- 7 sigma (:84-96); leading
  ``wrap`` / ``image`` keywords;
* default priors from plugin defaults (src/input/objects.c:225-226): a
  positive or negative-zero default becomes a delta prior;
* parameter bounds (src/lensed.c:140-171): the plugin's bounds, else [0, inf)
  for radii and [0, 1] for axis ratios; bounded when either bound is nonzero;
* the parameter map (src/lensed.c:240-262): free parameters in object order,
  then the derived (pseudo-prior) ones;
* the transform (src/nested.c:42-61): u = cube[i] for the free parameters and
  0.5 for the derived ones; a value outside the bounds is where the reference
  would redraw forever, flagged here as rejected.

The plugin tables (names, types, bounds, defaults) come in as an argument:
the fixture tests/golden/plugin_params.json holds the reference's own.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Dict, List, Sequence, Tuple

import numpy as np

RADIUS, AXIS_RATIO = 3, 5


@dataclass
class Prior:
    kind: str  # "delta" | "unif" | "norm" | "none"
    a: float = 0.0
    b: float = 0.0
    wrap: bool = False
    image: bool = False

    def lower(self) -> float:
        return {"delta": self.a, "unif": self.a, "norm": self.a - 7 * self.b}.get(self.kind, -math.inf)

    def upper(self) -> float:
        return {"delta": self.a, "unif": self.b, "norm": self.a + 7 * self.b}.get(self.kind, math.inf)


def parse_prior(spec: str) -> Prior:
    tok = spec.split()
    wrap = image = False
    while tok and tok[0] in ("wrap", "image"):
        wrap |= tok[0] == "wrap"
        image |= tok[0] == "image"
        tok = tok[1:]
    if not tok:
        return Prior("none", wrap=wrap, image=image)
    if len(tok) == 1:
        return Prior("delta", float(tok[0]), wrap=wrap, image=image)
    if tok[0] in ("unif", "norm") and len(tok) == 3:
        return Prior(tok[0], float(tok[1]), float(tok[2]), wrap=wrap, image=image)
    raise ValueError(f"invalid prior definition: {spec}")


def norm_quantile(u: float) -> float:
    """src/prior/norm.c:9-16, evaluated in double without contraction."""
    t = math.sqrt(-2.0 * math.log(u)) if u < 0.5 else math.sqrt(-2.0 * math.log(1 - u))
    t = t - ((0.010328 * t + 0.802853) * t + 2.515517) / (((0.001308 * t + 0.189269) * t + 1.432788) * t + 1.0)
    return -t if u < 0.5 else t


def apply(p: Prior, u: float) -> float:
    if p.kind == "delta":
        return p.a
    if p.kind == "unif":
        return p.a + u * (p.b - p.a)
    if p.kind == "norm":
        return p.a + p.b * norm_quantile(u)
    return math.nan


@dataclass
class Param:
    id: str
    type: int
    lower: float
    upper: float
    bounded: bool
    prior: Prior
    derived: bool


class ParamSpace:
    def __init__(self, objects: Sequence[Tuple[str, str, Dict[str, str]]], plugin_table: dict):
        self.params: List[Param] = []
        for oid, plugin, priors in objects:
            for name, ptype, lo, hi, defval in plugin_table[plugin]["params"]:
                pri = Prior("none")
                if defval > 0 or math.copysign(1.0, defval) < 0:
                    pri = Prior("delta", defval)
                if priors and name in priors:
                    pri = parse_prior(priors[name])
                if not lo and not hi:
                    if ptype == RADIUS:
                        lo, hi = 0.0, math.inf
                    elif ptype == AXIS_RATIO:
                        lo, hi = 0.0, 1.0
                self.params.append(Param(f"{oid}.{name}", ptype, lo, hi, bool(lo or hi), pri, pri.kind == "delta"))
        free = [i for i, p in enumerate(self.params) if not p.derived]
        self.ndims = len(free)
        self.pmap = free + [i for i, p in enumerate(self.params) if p.derived]

    @property
    def npars(self) -> int:
        return len(self.params)

    def transform(self, cube) -> Tuple[np.ndarray, np.ndarray]:
        """(B, ndims) unit cube -> ((B, npars) physical values in map order,
        (B,) rejected flags)."""
        cube = np.atleast_2d(np.asarray(cube, dtype=np.float64))
        B = cube.shape[0]
        out = np.empty((B, self.npars))
        bad = np.zeros(B, dtype=bool)
        for b in range(B):
            for i, k in enumerate(self.pmap):
                p = self.params[k]
                u = float(cube[b, i]) if i < self.ndims else 0.5
                v = apply(p.prior, u)
                if p.bounded and (v < p.lower or v > p.upper):
                    bad[b] = True
                out[b, i] = v
        return out, bad
