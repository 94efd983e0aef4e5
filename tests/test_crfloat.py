"""The correctly rounded single-precision exp, log, atan and atanh of the
exact evaluation modules, on the CPU.

lensed_gb300/device/lg_crfloat.cuh computes each function in
single-precision double-word arithmetic and rounds with Ziv's test, falling
back to the double evaluation where the test cannot decide.  Compiled for
the host (the same source with IEEE float operations and std::fma), every
result must equal the function evaluated in double and rounded once --
the oracle's semantics -- bit for bit.  Checked here on a stride through
all 2^32 bit patterns plus dense windows where the algorithms switch paths
(subnormal exp results, logarithms near 1, the two atanh formulas, atan
near 1); the whole range of all four functions was swept without a
mismatch when the code was written, and the GPU tests sweep it on the
device (test_gpu_crfloat.py).  The share of in-range inputs that need the
double path is bounded too (about 2^-15 to 2^-19).
"""
import os
import struct
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "native", "crf_sweep.cpp")


def bits(x):
    return struct.unpack("I", struct.pack("f", x))[0]


@pytest.fixture(scope="module")
def sweep(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("crf") / "crf_sweep")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp", SRC, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    def run(fn, start, stop, step=1):
        out = subprocess.run([exe, str(fn), str(start), str(stop), str(step)], capture_output=True, text=True,
                             timeout=600)
        assert out.returncode == 0, out.stderr
        n, bad, nin, slow = (int(v) for v in out.stdout.split())
        return n, bad, nin, slow, out.stderr

    return run


@pytest.mark.parametrize("fn,name", [(0, "exp"), (1, "log"), (2, "atan"), (3, "atanh")])
def test_stride_through_all_floats(sweep, fn, name):
    n, bad, nin, slow, err = sweep(fn, 0, 1 << 32, 257)
    print(f"{name}: {n} inputs, {bad} mismatches, {slow} of {nin} in range through double "
          f"({slow / max(nin, 1):.2g})")
    assert bad == 0, err
    assert slow <= 2.0 ** -13 * nin


WINDOWS = [
    (0, bits(-87.0), bits(-104.0)),          # exp: results below 2^-126 (negative floats grow in bits)
    (0, bits(-1e-3), bits(-0.5)),             # exp: small negative arguments
    (0, bits(80.0), bits(88.7)),              # exp: the largest k
    (1, bits(0.99), bits(1.01)),              # log near 1 (the c = 1 intervals and their neighbours)
    (1, bits(1.49), bits(1.51)),              # log at the exponent switch of the reduction
    (2, bits(0.97), bits(1.03)),              # atan around the reciprocal switch
    (2, bits(1e-4), bits(3e-3)),              # atan: the first table intervals
    (3, bits(0.05), bits(0.08)),              # atanh at the switch between its two formulas
    (3, bits(1e-4), bits(3e-3)),              # atanh: small arguments
    (3, bits(0.99), bits(1.0)),               # atanh near 1
]


@pytest.mark.parametrize("fn,lo,hi", WINDOWS)
def test_dense_windows(sweep, fn, lo, hi):
    lo, hi = min(lo, hi), max(lo, hi)
    n, bad, nin, slow, err = sweep(fn, lo, hi, 1 + (hi - lo) // 4000000)
    assert n > 100000 and bad == 0, err
