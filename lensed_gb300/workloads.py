"""Seeded synthetic lens systems for the benchmark and parity workloads.

No public dataset is involved: every image is a mock drawn from a fixed
numpy PCG64 seed.  The mock is rendered here in float64 numpy at 3x3
sub-pixel resolution (independently of the CUDA path and of the oracle),
convolved with the PSF, and given Poisson noise on model + sky plus Gaussian
read noise; weights follow Lensed's ``gain / (image + offset)``.

Coordinates are pixels (docs/units.md): 1.0 arcsec is 20 px at 0.05"/px and
50 px at 0.02"/px; the lens sits at the image centre (W+1)/2 +- 0.05".
Position angles are degrees in [0, 180).

Workloads (the model layouts are stated because the plugin parameter counts
fix them):

``small``   128^2, 0.05"/px, sie (5) + sersic (7) + sky (bg free), no PSF,
            9-point sub3 rule, B = 1.
``config2`` 256^2, 0.05"/px, sie_plus_shear (7) + sersic bulge (7) +
            exponential disk (6, the reference's exponential plugin) + sky
            (bg free, gradients fixed at 0): 23 parameters, 21 free;
            25x25 Gaussian-plus-wings PSF (FWHM 0.1" = 2 px), 25-point sub5
            rule, 10% random mask, B = 1024 per launch.
``systems`` 16 systems with sizes from {64, 128, 256, 512}^2, epl_plus_shear
            (slope t = gamma - 1, gamma ~ U[1.8, 2.2]) + sersic, odd PSFs
            15..31, g3k7 rule, 256 candidates per system.
``large``   1024^2, 0.02"/px, epl_plus_shear + nsie + point_mass lenses,
            sersic + sersic + gauss sources, sky; 41x41 PSF, 49-point g3k7
            rule, B = 256.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from math import lgamma, log, pi
from typing import List, Optional, Tuple

import numpy as np

__all__ = ["System", "make_system", "small", "config2", "systems", "large", "draw_candidates", "psf_gauss_wings"]


@dataclass
class System:
    name: str
    width: int
    height: int
    image: np.ndarray
    weight: np.ndarray
    psf: Optional[np.ndarray]
    rule: str
    objects: List[Tuple[str, str, dict]]  # (id, plugin, priors by parameter name)
    truth: np.ndarray                      # physical parameters in object order
    lower: np.ndarray                      # candidate box (object order)
    upper: np.ndarray
    pcs: Tuple[float, float, float, float] = (1.0, 1.0, 1.0, 1.0)
    mask: Optional[np.ndarray] = None
    meta: dict = field(default_factory=dict)

    @property
    def plugins(self):
        return [o[1] for o in self.objects]


# -------------------------------------------------------------- mock physics
def _rot(pa):
    c, s = np.cos(np.radians(pa)), np.sin(np.radians(pa))
    return c, s


def _sie(x1, x2, p, shear=None):
    x0, y0, r, q, pa = p[:5]
    c, s = _rot(pa)
    dx, dy = x1 - x0, x2 - y0
    y1, y2 = c * dx + s * dy, -s * dx + c * dy
    e = np.sqrt(1 - q * q)
    d = r * np.sqrt(q) / e
    rr = e / np.sqrt(q * q * y1 * y1 + y2 * y2)
    a1, a2 = d * np.arctan(y1 * rr), d * np.arctanh(np.clip(y2 * rr, -1 + 1e-15, 1 - 1e-15))
    ax, ay = c * a1 - s * a2, s * a1 + c * a2
    if shear is not None:
        g1, g2 = shear
        ax, ay = ax + g1 * dx + g2 * dy, ay + g2 * dx - g1 * dy
    return ax, ay


def _epl(x1, x2, p, shear=None):
    x0, y0, r, t, q, pa = p[:6]
    c, s = _rot(pa)
    dx, dy = x1 - x0, x2 - y0
    k = 1 / r / np.sqrt(q)
    u1, u2 = k * (q * c * dx + q * s * dy), k * (-s * dx + c * dy)
    R = np.hypot(u1, u2)
    phi = np.arctan2(u2, u1)
    f = (1 - q) / (1 + q)
    T = 2 - t
    A1, A2 = np.cos(phi), np.sin(phi)
    a1, a2 = A1.copy(), A2.copy()
    c2, s2 = np.cos(2 * phi), np.sin(2 * phi)
    for n in range(1, 11):
        co = -f * (2 * n - T) / (2 * n + T)
        A1, A2 = co * (c2 * A1 - s2 * A2), co * (s2 * A1 + c2 * A2)
        a1, a2 = a1 + A1, a2 + A2
    nrm = 2 * r * np.sqrt(q) / (1 + q) * np.power(np.maximum(R, 1e-30), 1 - t)
    a1, a2 = nrm * a1, nrm * a2
    ax, ay = c * a1 - s * a2, s * a1 + c * a2
    if shear is not None:
        g1, g2 = shear
        ax, ay = ax + g1 * dx + g2 * dy, ay + g2 * dx - g1 * dy
    return ax, ay


def _nsie(x1, x2, p):
    x0, y0, r, rc, q, pa = p
    c, s = _rot(pa)
    dx, dy = x1 - x0, x2 - y0
    y1, y2 = c * dx + s * dy, -s * dx + c * dy
    e = np.sqrt(1 - q * q)
    d = r * np.sqrt(q) / e
    rr = np.sqrt(q * q * y1 * y1 + y2 * y2)
    a1, a2 = d * np.arctan(y1 * e / (rc + rr)), d * np.arctanh(y2 * e / (rc * q * q + rr))
    return c * a1 - s * a2, s * a1 + c * a2


def _point_mass(x1, x2, p):
    x0, y0, r = p
    dx, dy = x1 - x0, x2 - y0
    d2 = np.maximum(dx * dx + dy * dy, 1e-12)
    return r * r / d2 * dx, r * r / d2 * dy


def _sersic(x1, x2, p):
    x0, y0, r, mag, n, q, pa = p
    b = 2 * n - 1 / 3 + 4 / (405 * n) + 46 / (25515 * n * n) + 131 / (1148175 * n ** 3) - 2194697 / (30690717750 * n ** 4)
    c, s = _rot(pa)
    dx, dy = x1 - x0, x2 - y0
    y1, y2 = (q * c * dx + q * s * dy) / np.sqrt(q), (-s * dx + c * dy) / np.sqrt(q)
    log0 = -0.4 * mag * log(10) + 2 * n * log(b) - log(pi) - 2 * log(r) - lgamma(2 * n + 1)
    log1 = log(b) - log(r) / n
    return np.exp(log0 - np.exp(log1 + 0.5 / n * np.log(np.maximum(y1 * y1 + y2 * y2, 1e-300))))


def _exponential(x1, x2, p):
    x0, y0, rs, mag, q, pa = p
    c, s = _rot(pa)
    dx, dy = x1 - x0, x2 - y0
    y1, y2 = q * c * dx + q * s * dy, -s * dx + c * dy
    norm = 10 ** (-0.4 * mag) * 0.5 / pi / rs / rs / q
    return norm * np.exp(-np.hypot(y1, y2) / rs)


def _gauss(x1, x2, p):
    x0, y0, sig, mag, q, pa = p
    c, s = _rot(pa)
    dx, dy = x1 - x0, x2 - y0
    y1, y2 = q * c * dx + q * s * dy, -s * dx + c * dy
    norm = 10 ** (-0.4 * mag) * 0.5 / pi / sig / sig / q
    return norm * np.exp(-0.5 * (y1 * y1 + y2 * y2) / sig / sig)


_LENS = {"sie": lambda x, y, p: _sie(x, y, p), "sie_plus_shear": lambda x, y, p: _sie(x, y, p, p[5:7]),
         "epl": lambda x, y, p: _epl(x, y, p), "epl_plus_shear": lambda x, y, p: _epl(x, y, p, p[6:8]),
         "nsie": _nsie, "point_mass": _point_mass}
_SRC = {"sersic": _sersic, "exponential": _exponential, "gauss": _gauss}
_NPARS = {"sie": 5, "sie_plus_shear": 7, "epl": 6, "epl_plus_shear": 8, "nsie": 6, "point_mass": 3, "sersic": 7,
          "exponential": 6, "gauss": 6, "sky": 3}


def mock_model(width, height, plugins, params, sub=3, pcs=(1.0, 1.0, 1.0, 1.0)):
    """Noise-free mock (float64), sub x sub point sampling per pixel."""
    off = (np.arange(sub) + 0.5) / sub - 0.5
    out = np.zeros((height, width))
    yy, xx = np.mgrid[0:height, 0:width].astype(np.float64)
    bx, by = pcs[0] + pcs[2] * xx, pcs[1] + pcs[3] * yy
    for ox in off:
        for oy in off:
            x1, x2 = bx + ox * pcs[2], by + oy * pcs[3]
            y1, y2 = x1.copy(), x2.copy()
            ax = np.zeros_like(x1); ay = np.zeros_like(x1)
            k = 0
            f = np.zeros_like(x1)
            for pl in plugins:
                p = params[k:k + _NPARS[pl]]
                k += _NPARS[pl]
                if pl in _LENS:
                    dxa, dya = _LENS[pl](x1, x2, p)
                    ax, ay = ax + dxa, ay + dya
                elif pl in _SRC:
                    f = f + _SRC[pl](x1 - ax, x2 - ay, p)
                elif pl == "sky":
                    f = f + p[0] + p[1] * (x1 - 1) + p[2] * (x2 - 1)
            out += f / (sub * sub)
    return out


def psf_gauss_wings(size: int, fwhm: float, wing_frac: float = 0.1, wing_scale: float = 4.0):
    """Normalised Gaussian core plus a broader Gaussian wing, odd or even size."""
    c = (size - 1) / 2
    yy, xx = np.mgrid[0:size, 0:size] - c
    r2 = xx * xx + yy * yy
    s = fwhm / 2.3548200450309493
    core = np.exp(-0.5 * r2 / s / s) / (2 * pi * s * s)
    sw = s * wing_scale
    wing = np.exp(-0.5 * r2 / sw / sw) / (2 * pi * sw * sw)
    p = (1 - wing_frac) * core + wing_frac * wing
    return (p / p.sum()).astype(np.float32)


def _convolve(img, psf):
    from scipy.signal import fftconvolve

    pad = max(psf.shape)
    big = np.pad(img, pad, mode="edge")
    return fftconvolve(big, psf, mode="same")[pad:-pad, pad:-pad]


def make_system(name, width, plugins, ids, truth, lower, upper, priors, rule, psf=None, sky=10.0, gain=1.0,
                read_noise=1.0, mask_frac=0.0, seed=0, height=None):
    height = height or width
    rng = np.random.Generator(np.random.PCG64(seed))
    model = mock_model(width, height, plugins, truth)
    if psf is not None:
        model = _convolve(model, psf.astype(np.float64))
    counts = rng.poisson(np.maximum(model * gain, 0)) / gain
    image = (counts + rng.normal(0.0, read_noise, size=model.shape)).astype(np.float32)
    offset = read_noise ** 2
    weight = (gain / (image.astype(np.float64) + offset)).astype(np.float32)
    weight[~np.isfinite(weight) | (weight < 0)] = 0
    mask = None
    if mask_frac > 0:
        mask = (rng.random(size=image.shape) < mask_frac).astype(np.int32)
        weight[mask != 0] = 0
    objects = [(i, p, pr) for i, p, pr in zip(ids, plugins, priors)]
    return System(name, width, height, image, weight, psf, rule, objects, np.asarray(truth, np.float64),
                  np.asarray(lower, np.float64), np.asarray(upper, np.float64), mask=mask,
                  meta={"sky": sky, "gain": gain, "read_noise": read_noise, "seed": seed})


def _box(truth, spans):
    t = np.asarray(truth, np.float64)
    s = np.asarray(spans, np.float64)
    return t - s, t + s


# Parameter names of the built-in plugins in their declaration order
# (objects/<name>.cl `params` blocks).  Kept in Python so that building a
# workload never loads the native library: the CPU reference arm of the
# bench must run without it.  tests/test_cabi.py checks this table against
# the library's plugin registry.
PLUGIN_PARAM_NAMES = {
    "sis": ("x", "y", "r"),
    "sis_plus_shear": ("x", "y", "r", "g1", "g2"),
    "nsis": ("x", "y", "r", "rc"),
    "sie": ("x", "y", "r", "q", "pa"),
    "sie_plus_shear": ("x", "y", "r", "q", "pa", "g1", "g2"),
    "nsie": ("x", "y", "r", "rc", "q", "pa"),
    "point_mass": ("x", "y", "r"),
    "epl": ("x", "y", "r", "t", "q", "pa"),
    "epl_plus_shear": ("x", "y", "r", "t", "q", "pa", "g1", "g2"),
    "sersic": ("x", "y", "r", "mag", "n", "q", "pa"),
    "sersic_old": ("x", "y", "r", "mag", "n", "q", "pa"),
    "exponential": ("x", "y", "rs", "mag", "q", "pa"),
    "devauc": ("x", "y", "r", "mag", "q", "pa"),
    "gauss": ("x", "y", "sigma", "mag", "q", "pa"),
    "sky": ("bg", "dx", "dy"),
}


def _priors_from_box(plugins, lower, upper, fixed):
    """Per-object dicts of prior strings: 'unif lo hi' or a fixed value."""
    out, k = [], 0
    for pl in plugins:
        names = PLUGIN_PARAM_NAMES[pl]
        d = {}
        for n in names:
            if k in fixed:
                d[n] = repr(float(fixed[k]))
            else:
                d[n] = f"unif {float(lower[k])!r} {float(upper[k])!r}"
            k += 1
        out.append(d)
    return out


def small(seed: int = 1) -> System:
    """128^2 SIE + Sersic + sky, no PSF, sub3 (9 points)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    W = 128
    c = (W + 1) / 2
    lx, ly = c + rng.uniform(-1, 1, 2)
    q, pa = rng.uniform(0.6, 0.95), rng.uniform(0, 180)
    n, re = rng.uniform(1, 4), rng.uniform(2, 8)
    sx, sy = lx + rng.uniform(-4, 4), ly + rng.uniform(-4, 4)
    sq, spa = rng.uniform(0.5, 0.95), rng.uniform(0, 180)
    mag = _mag_for_snr(30.0, re, n, sq, 10.0)
    truth = [lx, ly, 20.0, q, pa, sx, sy, re, mag, n, sq, spa, 10.0, -0.0, -0.0]
    spans = [1, 1, 2, 0.1, 20, 2, 2, 1, 0.5, 0.5, 0.1, 20, 1, 0, 0]
    lo, hi = _box(truth, spans)
    lo[3], hi[3] = max(lo[3], 0.3), min(hi[3], 0.99)
    lo[10], hi[10] = max(lo[10], 0.3), min(hi[10], 1.0)
    plugins = ["sie", "sersic", "sky"]
    pri = _priors_from_box(plugins, lo, hi, {13: -0.0, 14: -0.0})
    return make_system("small-128-sie-sersic-sky-q9", W, plugins, ["lens", "src", "sky"], truth, lo, hi, pri, "sub3",
                       seed=seed)


def _mag_for_snr(snr, re, n, q, sky):
    """Magnitude whose Sersic peak pixel has the given S/N over sky."""
    # peak surface brightness of the profile at the centre of one pixel
    b = 2 * n - 1 / 3 + 4 / (405 * n)
    target = snr * np.sqrt(sky) + snr * snr / 2  # counts per pixel at the peak
    log0_m0 = 2 * n * log(b) - log(pi) - 2 * log(re) - lgamma(2 * n + 1)
    peak0 = np.exp(log0_m0 - np.exp(log(b) - log(re) / n + 0.5 / n * log(0.25 / q)))
    return float(-2.5 * np.log10(target / peak0))


def config2(seed: int = 2) -> System:
    """Headline workload: 256^2 SIE+shear, bulge + disk, sky, 25^2 PSF, sub5."""
    rng = np.random.Generator(np.random.PCG64(seed))
    W = 256
    c = (W + 1) / 2
    lx, ly = c + rng.uniform(-1, 1, 2)
    lens = [lx, ly, 20.0, rng.uniform(0.6, 0.95), rng.uniform(0, 180), rng.uniform(0, 0.1) * np.cos(0.3),
            rng.uniform(0, 0.1) * np.sin(0.3)]
    sx, sy = lx + rng.uniform(-4, 4), ly + rng.uniform(-4, 4)
    n, re = rng.uniform(1, 4), rng.uniform(2, 8)
    bq = rng.uniform(0.5, 0.95)
    bulge = [sx, sy, re, _mag_for_snr(30.0, re, n, bq, 10.0), n, bq, rng.uniform(0, 180)]
    rs = rng.uniform(3, 8)
    disk = [sx, sy, rs, bulge[3] + 0.5, rng.uniform(0.4, 0.9), rng.uniform(0, 180)]
    truth = lens + bulge + disk + [10.0, -0.0, -0.0]
    spans = [1, 1, 2, 0.1, 20, 0.03, 0.03] + [2, 2, 1, 0.5, 0.5, 0.1, 20] + [2, 2, 1, 0.5, 0.1, 20] + [1, 0, 0]
    lo, hi = _box(truth, spans)
    for i in (3, 12, 18):
        lo[i], hi[i] = max(lo[i], 0.3), min(hi[i], 0.99)
    plugins = ["sie_plus_shear", "sersic", "exponential", "sky"]
    pri = _priors_from_box(plugins, lo, hi, {21: -0.0, 22: -0.0})
    psf = psf_gauss_wings(25, 2.0)
    return make_system("config2-256-siegamma-bulge-disk-sky-p25-q25", W, plugins, ["lens", "bulge", "disk", "sky"],
                       truth, lo, hi, pri, "sub5", psf=psf, mask_frac=0.10, seed=seed)


def systems(seed: int = 3, count: int = 16) -> List[System]:
    """Uneven batch: 16 systems, sizes from {64,128,256,512}^2, EPL+shear + Sersic."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for s in range(count):
        W = int(rng.choice([64, 128, 256, 512]))
        P = int(rng.choice(np.arange(15, 32, 2)))
        c = (W + 1) / 2
        er = W / 6.4
        lx, ly = c + rng.uniform(-1, 1, 2)
        lens = [lx, ly, er, rng.uniform(0.8, 1.2), rng.uniform(0.6, 0.95), rng.uniform(0, 180),
                rng.uniform(-0.05, 0.05), rng.uniform(-0.05, 0.05)]
        n, re = rng.uniform(1, 4), er * rng.uniform(0.1, 0.4)
        q = rng.uniform(0.5, 0.95)
        src = [lx + rng.uniform(-er / 5, er / 5), ly + rng.uniform(-er / 5, er / 5), re,
               _mag_for_snr(30.0, re, n, q, 10.0), n, q, rng.uniform(0, 180)]
        truth = lens + src + [10.0, -0.0, -0.0]
        spans = [1, 1, er / 10, 0.1, 0.1, 20, 0.02, 0.02, 2, 2, re / 5, 0.5, 0.5, 0.1, 20, 1, 0, 0]
        lo, hi = _box(truth, spans)
        lo[4], hi[4] = max(lo[4], 0.3), min(hi[4], 0.99)
        lo[13], hi[13] = max(lo[13], 0.3), min(hi[13], 0.99)
        plugins = ["epl_plus_shear", "sersic", "sky"]
        pri = _priors_from_box(plugins, lo, hi, {16: -0.0, 17: -0.0})
        out.append(make_system(f"system{s}-{W}-epl-sersic-p{P}", W, plugins, ["lens", "src", "sky"], truth, lo, hi,
                               pri, "g3k7", psf=psf_gauss_wings(P, 2.0), seed=seed * 100 + s))
    return out


def large(seed: int = 5) -> System:
    """1024^2 at 0.02"/px: EPL+shear + NSIE + point mass, 2 Sersic + Gauss, sky, P=41, g3k7."""
    rng = np.random.Generator(np.random.PCG64(seed))
    W = 1024
    c = (W + 1) / 2
    lx, ly = c + rng.uniform(-2.5, 2.5, 2)
    main = [lx, ly, 50.0, rng.uniform(0.8, 1.2), rng.uniform(0.6, 0.95), rng.uniform(0, 180),
            rng.uniform(-0.05, 0.05), rng.uniform(-0.05, 0.05)]
    sat = [lx + 60, ly - 30, 8.0, 1.0, rng.uniform(0.6, 0.95), rng.uniform(0, 180)]
    pert = [lx - 45, ly + 40, 2.0]
    s1 = [lx + 5, ly - 4, 10.0, 0.0, 2.5, 0.8, 30.0]
    s1[3] = _mag_for_snr(30.0, 10.0, 2.5, 0.8, 10.0)
    s2 = [lx - 8, ly + 6, 6.0, s1[3] + 1.0, 1.0, 0.6, 120.0]
    g = [lx + 2, ly + 12, 2.0, s1[3] + 2.0, 0.9, 10.0]
    truth = main + sat + pert + s1 + s2 + g + [10.0, -0.0, -0.0]
    spans = ([1, 1, 2, 0.05, 0.05, 10, 0.01, 0.01] + [1, 1, 0.5, 0.2, 0.05, 10] + [1, 1, 0.2] +
             [1, 1, 0.5, 0.3, 0.3, 0.05, 10] + [1, 1, 0.5, 0.3, 0.3, 0.05, 10] + [0.5, 0.5, 0.2, 0.3, 0.05, 10] +
             [0.5, 0, 0])
    lo, hi = _box(truth, spans)
    plugins = ["epl_plus_shear", "nsie", "point_mass", "sersic", "sersic", "gauss", "sky"]
    pri = _priors_from_box(plugins, lo, hi, {len(truth) - 2: -0.0, len(truth) - 1: -0.0})
    return make_system("large-1024-epl-nsie-pm-3src-sky-p41-q49", W, plugins,
                       ["lens", "sat", "pert", "src1", "src2", "clump", "sky"], truth, lo, hi, pri, "g3k7",
                       psf=psf_gauss_wings(41, 5.0), seed=seed)


def draw_candidates(sys: System, B: int, seed: int = 0, near: float = 0.5) -> np.ndarray:
    """B candidate vectors in object order: a fraction ``near`` within 10% of
    the box around the truth, the rest uniform in the box; fixed parameters
    keep their truth value."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lo, hi, t = sys.lower, sys.upper, sys.truth
    u = rng.random(size=(B, t.size))
    box = lo + u * (hi - lo)
    nb = int(B * near)
    box[:nb] = t + (box[:nb] - t) * 0.1
    fixed = lo == hi
    box[:, fixed] = t[fixed]
    return box
