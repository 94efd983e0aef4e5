"""Build liblensed_gb300.so (nvcc, sm_103a) in place.

Steps:
1. embed the device sources (``device/*.cuh`` and ``objects/*.cuh``) as C++
   raw strings into ``_build/lg_embed.inc`` -- they are composed per model
   and compiled with NVRTC at run time;
2. compile the host/CUDA translation units in parallel with
   ``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo``;
3. link ``lensed_gb300/liblensed_gb300.so`` against the static CUDA runtime
   and libnvrtc (the CUDA driver is resolved at run time, so the library
   also loads on machines without a GPU).
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "liblensed_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    raise RuntimeError("CUDA toolkit (nvcc) not found")


def _raw(text: str) -> str:
    assert ")LGRAW\"" not in text
    return 'R"LGRAW(' + text + ')LGRAW"'


def write_embed() -> str:
    os.makedirs(BUILD, exist_ok=True)
    prelude = open(os.path.join(PKG, "device", "lg_prelude.cuh")).read()
    kernels = open(os.path.join(PKG, "device", "lg_kernels.cuh")).read()
    setk = open(os.path.join(PKG, "device", "lg_set_kernel.cuh")).read()
    crmath = open(os.path.join(PKG, "device", "lg_crmath_on.cuh")).read()
    multi = open(os.path.join(PKG, "device", "lg_multi_kernels.cuh")).read()
    # the correctly rounded functions with their tables inlined (NVRTC has no
    # include path to this tree)
    inc = '#ifndef LG_CRF_TABLES_INLINE\n#include "lg_crf_tables.cuh"\n#endif\n'
    crf = open(os.path.join(PKG, "device", "lg_crfloat.cuh")).read()
    assert inc in crf
    crf = crf.replace(inc, open(os.path.join(PKG, "device", "lg_crf_tables.cuh")).read())
    exact = open(os.path.join(PKG, "device", "lg_exact_pair.cuh")).read()
    objs = sorted(glob.glob(os.path.join(PKG, "objects", "*.cuh")))
    lines = ["// generated by lensed_gb300/build.py: device sources for NVRTC", ""]
    lines.append(f"static const char LG_EMBED_PRELUDE[] = {_raw(prelude)};")
    lines.append(f"static const char LG_EMBED_KERNELS[] = {_raw(kernels)};")
    lines.append(f"static const char LG_EMBED_SET_KERNEL[] = {_raw(setk)};")
    lines.append(f"static const char LG_EMBED_CRMATH[] = {_raw(crmath)};")
    lines.append(f"static const char LG_EMBED_MULTI[] = {_raw(multi)};")
    lines.append(f"static const char LG_EMBED_CRF[] = {_raw(crf)};")
    lines.append(f"static const char LG_EMBED_EXACT_PAIR[] = {_raw(exact)};")
    lines.append("struct lg_embedded_object { const char* name; const char* text; };")
    lines.append("static const lg_embedded_object LG_EMBED_OBJECTS[] = {")
    for p in objs:
        name = os.path.splitext(os.path.basename(p))[0]
        lines.append(f'    {{"{name}", {_raw(open(p).read())}}},')
    lines.append("};")
    path = os.path.join(BUILD, "lg_embed.inc")
    text = "\n".join(lines) + "\n"
    if not os.path.exists(path) or open(path).read() != text:
        with open(path, "w") as f:
            f.write(text)
    return path


def sources():
    csrc = os.path.join(PKG, "csrc")
    return sorted(glob.glob(os.path.join(csrc, "*.cu")) + glob.glob(os.path.join(csrc, "*.cpp")))


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    write_embed()
    inc = ["-I", os.path.join(ROOT, "include"), "-I", BUILD, "-I", os.path.join(PKG, "csrc")]
    # host code: no floating-point contraction, so that it computes the same
    # bits on x86-64 and on aarch64 (where GCC would otherwise fuse a*b+c)
    flags = ["-O2", "-std=c++17", ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", "-Xcompiler",
             "-ffp-contract=off"]
    headers = glob.glob(os.path.join(PKG, "csrc", "*.h")) + glob.glob(os.path.join(PKG, "csrc", "*.inc")) + \
        glob.glob(os.path.join(PKG, "device", "*.cuh")) + glob.glob(os.path.join(PKG, "objects", "*.cuh")) + [
        os.path.join(ROOT, "include", "lensed_gb300.h"), os.path.join(BUILD, "lg_embed.inc")]
    objs = []
    jobs = []
    for s in sources():
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _newer(o, [s] + headers):
            jobs.append([nvcc, "-c", s, "-o", o] + flags + inc)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        for err in ex.map(run, jobs):
            if verbose and err:
                print(err, file=sys.stderr)
    if force or jobs or _newer(LIB, objs):
        lib64 = os.path.join(cuda, "lib64")
        run([nvcc, "-shared", ARCH, "-o", LIB] + objs + ["-L", lib64, "-lnvrtc", "-Xlinker", f"-rpath,{lib64}"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
