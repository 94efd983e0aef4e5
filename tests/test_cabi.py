"""The C-ABI library without a GPU: load, exports, registry, composition."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import lensed_gb300 as lg
from lensed_gb300 import quadrature

HEADER = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "lensed_gb300.h")

PLUGINS = {
    "sis": ("L", ["x", "y", "r"]), "sis_plus_shear": ("L", ["x", "y", "r", "g1", "g2"]),
    "nsis": ("L", ["x", "y", "r", "rc"]), "sie": ("L", ["x", "y", "r", "q", "pa"]),
    "sie_plus_shear": ("L", ["x", "y", "r", "q", "pa", "g1", "g2"]), "nsie": ("L", ["x", "y", "r", "rc", "q", "pa"]),
    "point_mass": ("L", ["x", "y", "r"]), "epl": ("L", ["x", "y", "r", "t", "q", "pa"]),
    "epl_plus_shear": ("L", ["x", "y", "r", "t", "q", "pa", "g1", "g2"]),
    "sersic": ("S", ["x", "y", "r", "mag", "n", "q", "pa"]), "sersic_old": ("S", ["x", "y", "r", "mag", "n", "q", "pa"]),
    "exponential": ("S", ["x", "y", "rs", "mag", "q", "pa"]), "devauc": ("S", ["x", "y", "r", "mag", "q", "pa"]),
    "gauss": ("S", ["x", "y", "sigma", "mag", "q", "pa"]), "sky": ("F", ["bg", "dx", "dy"]),
}


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lg_\w+|loglike)\s*\(", text)) - {"lg_ctx"})


def test_library_exports_every_declared_symbol(native):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(native, n), n


def test_plugin_registry_matches_reference_parameter_blocks(native):
    got = {n: (k, p) for n, k, p in lg.plugins()}
    assert set(got) == set(PLUGINS)
    for name, (kind, pars) in PLUGINS.items():
        assert got[name][0] == kind
        assert [p[0] for p in lg.plugin_params(name)] == pars
    # parameter types, bounds and defaults of a few entries
    sky = lg.plugin_params("sky")
    assert np.signbit(sky[1][4]) and sky[1][4] == 0  # dx default -0 (fixed)
    epl = dict((p[0], p) for p in lg.plugin_params("epl"))
    assert (epl["t"][2], epl["t"][3]) == (0.0, 2.0)
    assert epl["q"][1] == 5 and epl["pa"][1] == 6 and epl["x"][1] == 1


def test_workload_name_table_matches_registry(native):
    from lensed_gb300.workloads import PLUGIN_PARAM_NAMES

    assert set(PLUGIN_PARAM_NAMES) == set(PLUGINS)
    for name, names in PLUGIN_PARAM_NAMES.items():
        assert [p[0] for p in lg.plugin_params(name)] == list(names), name


def test_building_workloads_does_not_load_the_library():
    """The CPU reference arm of the bench builds its workload with no native
    code of the package mapped into the process."""
    import subprocess
    import sys

    code = ("import sys; sys.path.insert(0, '.'); import lensed_gb300 as lg; from lensed_gb300 import workloads; "
            "workloads.config2(); workloads.small(); workloads.large(); workloads.systems(); "
            "maps = open('/proc/self/maps').read(); print('liblensed_gb300' in maps, lg._lib is None)")
    root = os.path.dirname(os.path.dirname(__file__))
    out = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    assert out.stdout.split() == ["False", "True"], out.stdout


def test_library_rules_equal_python_rules(native):
    rules = lg.quad_rules()
    for name, (a, w, e) in rules.items():
        r = quadrature.rule(name)
        assert np.array_equal(a, np.array(r.points)), name
        assert np.array_equal(w, np.array(r.weights)), name
        assert np.array_equal(e, np.array(r.errors)), name


@pytest.mark.parametrize("plugin", sorted(PLUGINS))
def test_every_plugin_composes_for_sm103a(native, plugin):
    kind = PLUGINS[plugin][0]
    objs = [plugin] if kind != "S" else ["sie", plugin]
    if kind == "L":
        objs = [plugin, "sersic"]
    lg.compile_check(32, 32, objs, rule="sub2")


def test_composition_with_psf_ipp_and_strict_mode(native):
    psf = np.ones((6, 6), np.float32)  # even size: half-pixel shift path
    objs = [("host", "sersic", None), ("lens", "sie_plus_shear", None),
            ("src", "sersic", {"x": "image unif 10 12", "y": "image unif 10 12", "r": "1", "mag": "0", "n": "2",
                                "q": "0.7", "pa": "10"}), ("sky", "sky", None)]
    lg.compile_check(40, 30, objs, psf=psf, rule="gm75")
    lg.compile_check(40, 30, objs, psf=psf, rule="gm75", flags=lg.LG_FLAG_STRICT_FP)


def test_invalid_models_are_rejected_with_status(native):
    with pytest.raises(lg.LensedError) as e:
        lg.compile_check(10, 10, ["nonexistent"])
    assert e.value.code == -1
    with pytest.raises(lg.LensedError) as e:
        lg.compile_check(10, 10, ["sie", "sersic", "sis", "sersic"])  # two lens planes
    assert e.value.code == -6
    with pytest.raises(lg.LensedError):
        lg.compile_check(10, 10, ["sie", "sersic"], rule="nope")
    with pytest.raises(lg.LensedError):  # bad prior syntax
        lg.compile_check(10, 10, [("l", "sie", {"x": "unif 1", "y": "1", "r": "1", "q": "0.5", "pa": "0"})])
    with pytest.raises(lg.LensedError):  # image-plane prior on a radius
        lg.compile_check(10, 10, [("l", "sie", {"x": "1", "y": "1", "r": "image unif 1 2", "q": "0.5", "pa": "0"})])
    with pytest.raises(lg.LensedError):  # prior entirely outside the bounds (q in [0, 1])
        lg.compile_check(10, 10, [("l", "sie", {"x": "1", "y": "1", "r": "1", "q": "unif 2 3", "pa": "0"})])
    with pytest.raises(lg.LensedError):  # missing prior when priors are given
        lg.compile_check(10, 10, [("l", "sie", {"x": "1", "y": "1", "r": "1", "q": "0.5"})])


def test_register_plugin_extends_the_surface(native):
    src = b"""
struct lg_data_ring_test { float2 x; float r, w, a; };
LG_DEV void lg_set_ring_test(lg_data_ring_test* o, float x, float y, float r, float w, float a)
{ o->x = make_float2(x, y); o->r = r; o->w = w; o->a = a; }
LG_DEV float lg_brightness_ring_test(const lg_data_ring_test* __restrict__ o, float2 x)
{ float d = (length(x - o->x) - o->r) / o->w; return o->a * expf(-0.5f * d * d); }
"""

    class Desc(C.Structure):
        _fields_ = [("name", C.c_char_p), ("kind", C.c_int), ("npars", C.c_int), ("par_names", C.POINTER(C.c_char_p)),
                    ("par_types", C.POINTER(C.c_int)), ("par_bounds", C.POINTER(C.c_float)),
                    ("par_defaults", C.POINTER(C.c_float)), ("source", C.c_char_p)]

    names = (C.c_char_p * 5)(b"x", b"y", b"r", b"w", b"a")
    types = (C.c_int * 5)(1, 2, 3, 3, 0)
    d = Desc(b"ring_test", ord("S"), 5, names, types, None, None, src)
    native.lg_register_plugin.argtypes = [C.POINTER(Desc)]
    assert native.lg_register_plugin(C.byref(d)) == 0
    assert native.lg_register_plugin(C.byref(d)) == -1  # duplicate
    assert [p[0] for p in lg.plugin_params("ring_test")] == ["x", "y", "r", "w", "a"]
    lg.compile_check(16, 16, ["sie", "ring_test"], rule="point")


@pytest.mark.parametrize("name", ["small", "config2", "large"])
def test_benchmark_workloads_compose(native, name):
    """The seeded benchmark systems (priors included) compose and compile."""
    from lensed_gb300 import workloads

    s = getattr(workloads, name)()
    lg.compile_check(s.width, s.height, s.objects, psf=s.psf, rule=s.rule)


def test_systems_program_composes_without_gpu(native):
    """lg_systems_create compiles its programs before touching the GPU: on a
    machine without one it must fail with a CUDA error, not a compile error."""
    from lensed_gb300 import workloads
    import torch

    if torch.cuda.is_available():
        pytest.skip("GPU present: covered by the GPU tests")
    syst = workloads.systems(count=3)
    with pytest.raises(lg.LensedError) as e:
        lg.Systems([(s.image, s.weight, s.psf, None) for s in syst], syst[0].objects, capacity=[4, 4, 4])
    assert e.value.code == -3, str(e.value)
