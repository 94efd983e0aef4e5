"""The correctly rounded single-precision exp, log, atan, atanh, sin, cos,
pow and atan2 of the exact evaluation modules, on the CPU.

lensed_gb300/device/lg_crfloat.cuh computes each function in
single-precision double-word arithmetic and rounds with Ziv's test, falling
back to the double evaluation where the test cannot decide.  Compiled for
the host (the same source with IEEE float operations and std::fma), every
result must equal the function evaluated in double and rounded once --
the oracle's semantics -- bit for bit.  Checked here on a stride through
all 2^32 bit patterns plus dense windows where the algorithms switch paths
(subnormal exp results, logarithms near 1, the two atanh formulas, atan
near 1, sin and cos near multiples of pi/2, pow near 1); the whole range of
every function (for pow and atan2 every first argument, with a second
argument derived from it) was swept without a mismatch when the code was
written, and the GPU tests sweep it on the device (test_gpu_crfloat.py).  The share of in-range inputs that need the
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


# (fn, name, bound on the share of in-range inputs through double: pow's
# rounding-test margin grows with |y ln x|)
FUNCTIONS = [(0, "exp", -13), (1, "log", -13), (2, "atan", -13), (3, "atanh", -13), (4, "sin", -13),
             (5, "cos", -13), (6, "pow(x, fixed y)", -10), (7, "atan2(x, p)", -13), (8, "pow(|x|, p)", -10)]


@pytest.mark.parametrize("fn,name,slow_bound", FUNCTIONS)
def test_stride_through_all_floats(sweep, fn, name, slow_bound):
    n, bad, nin, slow, err = sweep(fn, 0, 1 << 32, 257 if fn < 4 else 1031)
    print(f"{name}: {n} inputs, {bad} mismatches, {slow} of {nin} in range through double "
          f"({slow / max(nin, 1):.2g})")
    assert bad == 0, err
    assert slow <= 2.0 ** slow_bound * nin


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
    (3, bits(0.89), bits(0.91)),              # atanh at the switch from the table to the logarithm
    (4, bits(1e-4), bits(0.02)),              # sin: small arguments, the first table intervals
    (4, bits(3.13), bits(3.16)),              # sin near pi (results near zero, k = 2)
    (5, bits(1.56), bits(1.58)),              # cos near pi/2
    (5, bits(127.0), bits(128.5)),            # cos at the end of the reduced range
    (6, bits(0.99), bits(1.01)),              # pow near x = 1 (y ln x near zero)
    (6, bits(1e-3), bits(200.0)),             # pow over the EPL lens's radii
    (7, bits(0.5), bits(2.0)),                # atan2 with arguments of similar size
    (8, bits(0.9), bits(1.1)),                # pow(|x|, p) near |x| = 1
]


@pytest.mark.parametrize("fn,lo,hi", WINDOWS)
def test_dense_windows(sweep, fn, lo, hi):
    lo, hi = min(lo, hi), max(lo, hi)
    n, bad, nin, slow, err = sweep(fn, lo, hi, 1 + (hi - lo) // 4000000)
    assert n > 100000 and bad == 0, err
