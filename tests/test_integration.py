"""The reference-side binding (include/lensed_gb300_lensed.h) compiled
against Lensed's own headers and prior code, on the CPU.

tests/native/lensed_binding_check.c builds a Lensed `input` whose priors
come from the reference's prior_read() (src/prior.c and src/prior/*.c,
compiled where they lie in the reference tree, LENSED_SOURCE), converts it
with the binding into the library's object list and asks the library to
compose and compile the model.  The prior strings must carry the
reference's wrap/image flags and its values (uniform bounds and fixed
values exactly, normal priors within an ulp).  Skipped where the reference
sources are absent."""
import os
import subprocess

import pytest

from oracle.build_ref import REF

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(REF, "src")


@pytest.mark.skipif(not os.path.isfile(os.path.join(SRC, "input.h")), reason="reference sources not present")
def test_binding_compiles_against_the_reference_and_composes(native, tmp_path):
    exe = str(tmp_path / "binding_check")
    libdir = os.path.join(ROOT, "lensed_gb300")
    srcs = [os.path.join(HERE, "native", "lensed_binding_check.c")] + [
        os.path.join(SRC, f) for f in ("prior.c", "prior/unif.c", "prior/norm.c", "prior/delta.c", "parse.c", "log.c")]
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", SRC, "-I", os.path.join(ROOT, "include")] + srcs +
                       ["-L", libdir, "-llensed_gb300", f"-Wl,-rpath,{libdir}", "-lm", "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
    got = dict(line.split(" = ", 1) for line in out.stdout.splitlines() if " = " in line)
    assert got["lens.x"] == "unif 20.25 28.125"
    assert got["lens.pa"] == "wrap unif 0 180"
    assert got["src.x"] == "image unif 10 20"
    assert got["sky.bg"] == "10.5"
    assert got["sky.dx"] == "(default)"
    kind, m, s = got["src.n"].split()
    assert kind == "norm" and float(m) == 2.5 and abs(float(s) - 0.1234567890123) <= 4e-17
    assert out.stdout.splitlines()[-1].startswith("lg_compile_check 0")
