"""Build the reference-built checker under oracle/_ref -- TEST INFRASTRUCTURE.

Compiles Lensed's own likelihood code for the host CPU, from the reference
source tree where it lies (LENSED_SOURCE, default /root/reference):

1. ``ref_gen`` = oracle/ref_gen.c + the reference's src/kernel.c (gcc): the
   reference's own program generator;
2. per object plugin, the reference's introspection program
   (object_program) is turned into C++ through oracle/clcompat.h to read the
   plugin's data size and parameter types (the values the reference reads
   back from the device in src/input/objects.c:110-190);
3. per model configuration, main_program() -- plugins, generated compute()
   and set_params, kernel/lensed.cl -- with kernel_options() as #defines, is
   turned into C++ and compiled with oracle/ref_harness.inc into
   oracle/_ref/<config>_{cr,libm}.so.

The only text changes are the mechanical ones C++ needs: ``(float2)(a, b)``
-> ``float2(a, b)`` (also float4/mat22), the read-only float4 halves
``.lo/.hi/.xy/.zw`` -> ``.lo()`` etc., and ``(local void*)`` ->
``(lg_anyptr)``; everything else is compiled as written.  Generated sources
stay in oracle/_ref/src (git-ignored) so a machine without the reference tree
can rebuild the libraries from them (``build_from_sources``).

Usage: python oracle/build_ref.py            # the standard configurations
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import subprocess
import sys
from typing import Dict, List, Sequence, Tuple

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
REF = os.environ.get("LENSED_SOURCE", "/root/reference")
CXX = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-w"]


def _run(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, text=True, **kw)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(cmd)}\n{r.stdout[-3000:]}\n{r.stderr[-3000:]}")
    return r.stdout


def to_cpp(text: str) -> str:
    for t in ("float2", "float4", "mat22"):
        text = text.replace(f"({t})(", f"{t}(")
    # float4 halves are read-only accessors in C++
    text = re.sub(r"\.(lo|hi|xy|zw)\b", r".\1()", text)
    return text.replace("(local void*)", "(lg_anyptr)")


def ref_gen() -> str:
    exe = os.path.join(OUT, "ref_gen")
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(HERE, "ref_gen.c"), os.path.join(REF, "src", "kernel.c")]
    if not os.path.exists(exe) or any(os.path.getmtime(s) > os.path.getmtime(exe) for s in srcs):
        _run(["gcc", "-std=gnu99", "-O1", "-w", "-U_FORTIFY_SOURCE", "-D_FORTIFY_SOURCE=0", "-fno-builtin",
              "-I", os.path.join(REF, "src"), "-o", exe] + srcs + ["-lm"])
    return exe


def _gen(*args) -> str:
    env = dict(os.environ, LENSED_SOURCE=REF.rstrip("/") + "/")
    return subprocess.run([ref_gen()] + [str(a) for a in args], capture_output=True, text=True, env=env,
                          check=True).stdout


_META: Dict[str, Tuple[str, int, List[int]]] = {}


def meta(name: str) -> Tuple[str, int, List[int]]:
    """(type, data size in floats, parameter types) of a reference object."""
    if name in _META:
        return _META[name]
    text = to_cpp(_gen("meta", name))
    # the params_ kernel reads names with vload16; only the table is needed
    text = re.sub(r"kernel void params_\w+\(.*?\n\}\n", "", text, flags=re.S)
    os.makedirs(SRC, exist_ok=True)
    cpp = os.path.join(SRC, f"meta_{name}.cpp")
    with open(cpp, "w") as f:
        f.write('#include <cstdio>\n#include "clcompat.h"\nthread_local size_t ref_gid[2], ref_grp[2];\n')
        f.write("namespace ref {\n" + text + "\n}\n#undef this\n#undef constant\n")
        f.write("int main() { int t; ulong s, n; ref::meta_%s(&t, &s, &n);\n" % name)
        f.write('  printf("%c %lu %lu", t, s, n);\n')
        f.write("  for (ulong i = 0; i < n; ++i) printf(\" %%d\", ref::parlst_%s[i].type);\n" % name)
        f.write("  printf(\"\\n\"); return 0; }\n")
    exe = cpp[:-4]
    _run(["g++", "-std=c++17", "-O0", "-w", "-I", HERE, "-o", exe, cpp])
    out = _run([exe]).split()
    t, size_bytes, n = out[0], int(out[1]), int(out[2])
    types = [int(v) for v in out[3:3 + n]]
    res = (t, (size_bytes + 3) // 4, types)  # rounded up to floats, src/input/objects.c:139
    _META[name] = res
    return res


def config_name(objects: Sequence[Tuple[str, int]], width: int, height: int, psf: Tuple[int, int], nq: int) -> str:
    key = json.dumps([list(map(list, objects)), width, height, list(psf), nq])
    return "cfg_" + hashlib.sha1(key.encode()).hexdigest()[:12]


def generate(objects: Sequence[Tuple[str, int]], width: int, height: int, psf: Tuple[int, int], nq: int) -> str:
    """Write the C++ source of one configuration; returns its base name."""
    name = config_name(objects, width, height, psf, nq)
    args = [width, height, 1 if psf[0] else 0, psf[0], psf[1], nq, len(objects)]
    dsiz = npars = 0
    for obj, ipp in objects:
        t, size, types = meta(obj)
        args += [obj, t, size, ",".join(map(str, types)), int(bool(ipp))]
        dsiz += size
        npars += len(types)
    text = _gen("main", *args)
    defines, body = text.split("//@@program@@\n", 1)
    body = to_cpp(body)
    os.makedirs(SRC, exist_ok=True)
    with open(os.path.join(SRC, name + ".cpp"), "w") as f:
        f.write("// generated by oracle/build_ref.py from the reference's own sources\n")
        f.write("#include <algorithm>\n#include <vector>\n#include \"clcompat.h\"\n")
        f.write(defines)
        f.write(f"#define REF_DSIZ {dsiz}\n#define REF_NPARS {npars}\n")
        f.write("namespace ref {\n" + body + "\n}\n")
        f.write('#include "ref_harness.inc"\n')
    with open(os.path.join(SRC, name + ".json"), "w") as f:
        json.dump({"objects": [list(o) for o in objects], "width": width, "height": height, "psf": list(psf),
                   "nq": nq}, f)
    return name


def compile_config(name: str) -> None:
    src = os.path.join(SRC, name + ".cpp")
    deps = [src, os.path.join(HERE, "clcompat.h"), os.path.join(HERE, "ref_harness.inc")]
    for mode, cr in (("cr", 1), ("libm", 0)):
        lib = os.path.join(OUT, f"{name}_{mode}.so")
        if os.path.exists(lib) and all(os.path.getmtime(d) <= os.path.getmtime(lib) for d in deps):
            continue
        _run(CXX + [f"-DREF_CR={cr}", "-I", HERE, "-o", lib, src])


def compile_all(names) -> None:
    from concurrent.futures import ThreadPoolExecutor

    with ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1))) as ex:
        list(ex.map(compile_config, sorted(set(names))))


def build_from_sources() -> int:
    """Compile every generated configuration found under oracle/_ref/src."""
    if not os.path.isdir(SRC):
        return 0
    names = [f[:-4] for f in sorted(os.listdir(SRC)) if f.startswith("cfg_") and f.endswith(".cpp")]
    compile_all(names)
    return len(names)


def standard_configs():
    """The configurations the tests and the benchmark use."""
    sys.path.insert(0, ROOT)
    from lensed_gb300 import quadrature, workloads

    out = []
    # reference test images (100x100, g3k7), plugins the reference can build
    fx = os.path.join(ROOT, "tests", "golden", "fixtures.npz")
    import numpy as np

    g = np.load(fx)
    for case in g["cases"]:
        plugins = [str(p) for p in g[f"{case}__plugins"]]
        if "sersic_old" in plugins:
            plugins = ["sersic" if p == "sersic_old" else p for p in plugins]
        out.append(([(p, 0) for p in plugins], 100, 100, (0, 0), quadrature.rule("g3k7").size))
    for s in (workloads.small(), workloads.config2()):
        psf = s.psf.shape[::-1] if s.psf is not None else (0, 0)
        out.append(([(p, 0) for p in s.plugins], s.width, s.height, psf, quadrature.rule(s.rule).size))
    # image-plane prior and even PSF cases of the parity tests
    out.append(([("sie", 0), ("sersic", 1)], 48, 48, (0, 0), 9))
    out.append(([("sie_plus_shear", 0), ("gauss", 0)], 45, 52, (7, 8), 4))
    return out


def main() -> None:
    if not os.path.isdir(os.path.join(REF, "src")):
        n = build_from_sources()
        print(f"reference tree not found; compiled {n} generated configurations")
        return
    names = []
    for objects, w, h, psf, nq in standard_configs():
        names.append(generate(objects, w, h, psf, nq))
    compile_all(names)
    print(f"built {len(set(names))} reference configurations in {OUT}")


if __name__ == "__main__":
    main()
