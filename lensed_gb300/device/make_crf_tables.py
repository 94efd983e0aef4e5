"""Generate lg_crf_tables.cuh: the tables and split constants of the
correctly rounded single-precision functions in lg_crfloat.cuh.

Every value is computed with mpmath at 60 significant digits and rounded to
float (round to nearest even) once; a "double-word" pair (hi, lo) holds
hi = RN(v) and lo = RN(v - hi).

  exp   T_j = 2^(j/64), j = 0..63, as (hi, lo)                (Tang 1989)
  log   for the 1024 intervals of the mantissa m in [0.75, 1.5) (512 of
        width 2^-11 below 1, 512 of width 2^-10 above): c_j = RN(1 / centre)
        (c = 1 for the two intervals next to 1) and -ln(c_j) as (hi, lo)
        (Tang 1990)
  atan  atan(j/512), j = 0..512, as (hi, lo)
  atanh atanh(j/512), j = 0..461, as (hi, lo)
  sin/cos  sin(j/256) and cos(j/256), j = -201..201, as (hi, lo) pairs

Run:  python lensed_gb300/device/make_crf_tables.py
"""
import os
import struct

import mpmath as mp

mp.mp.dps = 60
HERE = os.path.dirname(os.path.abspath(__file__))


def rn(v) -> float:
    """Round an mpmath value to the nearest float32 (ties to even)."""
    d = float(v)  # nearest double; re-round with the exact remainder
    f = struct.unpack("f", struct.pack("f", d))[0]
    # struct rounds the double to float with ties-to-even; correct a double
    # rounding by comparing against the exact value
    if f != 0 and mp.isfinite(v):
        lo_n = struct.unpack("f", struct.pack("I", struct.unpack("I", struct.pack("f", f))[0] - 1))[0]
        hi_n = struct.unpack("f", struct.pack("I", struct.unpack("I", struct.pack("f", f))[0] + 1))[0]
        best = min((abs(mp.mpf(c) - v), c) for c in (lo_n, f, hi_n))
        f = best[1]
    return f


def split(v):
    hi = rn(v)
    lo = rn(v - mp.mpf(hi))
    return hi, lo


def lit(f: float) -> str:
    if f == 0:
        return "0.0f"
    h = float.hex(f)  # e.g. 0x1.5d58980000000p-1
    mant, exp = h.split("p")
    if "." in mant:
        mant = mant.rstrip("0").rstrip(".")
    return f"{mant}p{exp}f"


def main():
    out = ["// generated by lensed_gb300/device/make_crf_tables.py -- do not edit",
           "// Tables of the correctly rounded single-precision functions (lg_crfloat.cuh).", ""]
    # exp: 2^(j/64)
    rows = []
    for j in range(64):
        hi, lo = split(mp.power(2, mp.mpf(j) / 64))
        rows.append(f"{{{lit(hi)}, {lit(lo)}}}")
    out.append("LG_CRF_TABLE(float2, lg_crf_exp_tab, 64) = {\n    " + ",\n    ".join(rows) + "};")
    # log: (c, -ln c hi, -ln c lo, 0)
    rows = []
    for j in range(1024):
        if j < 512:
            m0, w = mp.mpf(0.75) + j * mp.mpf(2) ** -11, mp.mpf(2) ** -11
        else:
            m0, w = 1 + (j - 512) * mp.mpf(2) ** -10, mp.mpf(2) ** -10
        c = 1.0 if j in (511, 512) else rn(1 / (m0 + w / 2))
        hi, lo = split(-mp.log(mp.mpf(c)))
        rows.append(f"{{{lit(c)}, {lit(hi)}, {lit(lo)}, 0.0f}}")
    out.append("LG_CRF_TABLE(float4, lg_crf_log_tab, 1024) = {\n    " + ",\n    ".join(rows) + "};")
    # atan(j/512)
    rows = []
    for j in range(513):
        hi, lo = split(mp.atan(mp.mpf(j) / 512))
        rows.append(f"{{{lit(hi)}, {lit(lo)}}}")
    out.append("LG_CRF_TABLE(float2, lg_crf_atan_tab, 513) = {\n    " + ",\n    ".join(rows) + "};")
    # atanh(j/512), j = 0..461, as (hi, lo)
    rows = []
    for j in range(462):
        hi, lo = split(mp.atanh(mp.mpf(j) / 512))
        rows.append(f"{{{lit(hi)}, {lit(lo)}}}")
    out.append("LG_CRF_TABLE(float2, lg_crf_atanh_tab, 462) = {\n    " + ",\n    ".join(rows) + "};")
    # sin / cos(j/256), j = -201..201, as (sin hi, sin lo, cos hi, cos lo)
    rows = []
    for j in range(-201, 202):
        a = mp.mpf(j) / 256
        sh, sl = split(mp.sin(a))
        ch, cl = split(mp.cos(a))
        rows.append(f"{{{lit(sh)}, {lit(sl)}, {lit(ch)}, {lit(cl)}}}")
    out.append("LG_CRF_TABLE(float4, lg_crf_sc_tab, 403) = {\n    " + ",\n    ".join(rows) + "};")
    # split constants
    consts = {}
    l64 = mp.log(2) / 64
    consts["LG_CRF_EXP_INVL"] = rn(64 / mp.log(2))
    consts["LG_CRF_EXP_LHI"], consts["LG_CRF_EXP_LLO"] = split(l64)
    consts["LG_CRF_LN2_HI"], consts["LG_CRF_LN2_LO"] = split(mp.log(2))
    consts["LG_CRF_PIO2_HI"], consts["LG_CRF_PIO2_LO"] = split(mp.pi / 2)
    # sin / cos argument reduction: 2/pi, and pi/2 = P1 + P2 + P3 with P1
    # and P2 of 17 significant bits (k P1, k P2 exact for |k| < 2^7)
    consts["LG_CRF_INV_PIO2"] = rn(2 / mp.pi)
    p1 = mp.floor(mp.pi / 2 * 2 ** 16 + mp.mpf(0.5)) / 2 ** 16
    p2 = mp.floor((mp.pi / 2 - p1) * 2 ** 33 + mp.mpf(0.5)) / 2 ** 33
    consts["LG_CRF_PIO2_1"], consts["LG_CRF_PIO2_2"] = rn(p1), rn(p2)
    assert mp.mpf(rn(p1)) == p1 and mp.mpf(rn(p2)) == p2
    consts["LG_CRF_PIO2_3"] = rn(mp.pi / 2 - p1 - p2)
    # exp(x) rounds to 0 for x <= LG_CRF_EXP_ZERO (e^x <= 2^-150, the tie at
    # 2^-150 going to the even value 0): the largest such float
    t = mp.log(mp.mpf(2) ** -150)
    f = rn(t)
    if mp.mpf(f) > t:  # e^f > 2^-150: step one float down (away from zero)
        f = struct.unpack("f", struct.pack("I", struct.unpack("I", struct.pack("f", f))[0] + 1))[0]
    consts["LG_CRF_EXP_ZERO"] = f
    for k, v in consts.items():
        out.append(f"#define {k} ({lit(v)})")
    text = "\n".join(out) + "\n"
    with open(os.path.join(HERE, "lg_crf_tables.cuh"), "w") as fh:
        fh.write(text)
    print(f"wrote {len(text)} bytes")


if __name__ == "__main__":
    main()
