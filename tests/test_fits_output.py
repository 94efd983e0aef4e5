"""FITS output of the dumper's layers (src/data.c:129-165, 372-419) and the
oracle's restatement of the layers (src/nested.c:217-254), on the CPU.

The writer is host code in the C-ABI library; it is read back with the
package's own FITS reader and checked card by card against the FITS fixed
format."""
import math
import os

import numpy as np
import pytest

import lensed_gb300 as lg
from lensed_gb300 import fits
from oracle.oracle import DUMP_NAMES, dump_layers


def _layers(W=37, H=23, n=6, seed=3):
    rng = np.random.default_rng(seed)
    out = [rng.normal(size=(H, W)).astype(np.float32) for _ in range(max(n, 5))]
    out[1][0, 0] = np.nan
    out[2][1, 2] = np.inf
    out[3][4, 5] = -0.0
    out[4][H - 1, W - 1] = np.float32(1e-40)  # subnormal
    return out[:n]


def _cards(block: bytes):
    return [block[i : i + 80].decode("ascii") for i in range(0, len(block), 80)]


def test_write_fits_roundtrip(native, tmp_path):
    layers = _layers()
    path = str(tmp_path / "out.fits")
    lg.write_fits(path, layers, list(DUMP_NAMES))
    raw = open(path, "rb").read()
    assert len(raw) % 2880 == 0
    hdus = fits.read_hdus(path)
    assert len(hdus) == 7
    prim = hdus[0]
    assert prim.header["SIMPLE"] is True and prim.header["NAXIS"] == 0 and prim.data is None
    assert prim.header["EXTEND"] is True and prim.header["ORIGIN"].startswith("lensed_gb300")
    for h, a, name in zip(hdus[1:], layers, DUMP_NAMES):
        assert h.header["XTENSION"] == "IMAGE" and h.header["BITPIX"] == -32
        assert (h.header["NAXIS1"], h.header["NAXIS2"]) == (37, 23)
        assert h.header["PCOUNT"] == 0 and h.header["GCOUNT"] == 1
        assert h.name == name
        assert np.array_equal(h.data.view(np.uint32), a.view(np.uint32))  # bit-exact incl. NaN, -0, subnormal


def test_cards_follow_fixed_format(native):
    b = lg.fits_bytes(_layers(n=1), ["IMG"])
    prim = _cards(b[:2880])
    assert prim[0] == "SIMPLE  =                    T / file does conform to FITS standard".ljust(80)
    assert prim[1].startswith("BITPIX  =                   16 /")
    end = [i for i, c in enumerate(prim) if c.rstrip() == "END"]
    assert len(end) == 1 and all(c == " " * 80 for c in prim[end[0] + 1 :])
    date = [c for c in prim if c.startswith("DATE    = '")][0]
    assert date[11:30][4] == "-" and date[11:30][10] == "T" and date[30] == "'"
    ext = _cards(b[2880 : 2 * 2880])
    assert ext[0].startswith("XTENSION= 'IMAGE   '")
    assert ext[1].startswith("BITPIX  =                  -32 /")
    assert ext[3].startswith("NAXIS1  =                   37 /")
    assert [c for c in ext if c.startswith("EXTNAME")][0].startswith("EXTNAME = 'IMG     '")
    # data: 37*23 float32 padded with zeros to a whole record
    data = b[2 * 2880 :]
    nbytes = 37 * 23 * 4
    assert len(data) == 2 * 2880 and data[nbytes:] == b"\0" * (2 * 2880 - nbytes)


def test_memory_matches_file(native, tmp_path):
    layers = _layers(W=64, H=64, n=3)
    names = ["A", None, "a quote ' here"]
    path = str(tmp_path / "m.fits")
    lg.write_fits(path, layers, names)
    mem = lg.fits_bytes(layers, names)
    disk = open(path, "rb").read()
    assert len(mem) == len(disk)
    strip = lambda b: b"".join(c for c in (b[i : i + 80] for i in range(0, len(b), 80)) if not c.startswith(b"DATE"))
    assert strip(mem) == strip(disk)
    hdus = fits.read_hdus(path)
    assert [h.name for h in hdus[1:]] == ["A", "", "a quote ' here"]
    # the reader's first-image rule picks the model layer of an output file
    img, pcs = fits.read_image(path)
    assert np.array_equal(img, layers[0]) and pcs == (1.0, 1.0, 1.0, 1.0)


def test_write_fits_errors(native, tmp_path):
    a = np.zeros((4, 4), np.float32)
    with pytest.raises(lg.LensedError):
        lg.write_fits(str(tmp_path / "x.fits"), [a], ["café"])
    with pytest.raises(lg.LensedError):
        lg.write_fits(str(tmp_path / "x.fits"), [a], ["N" * 69])
    with pytest.raises(lg.LensedError):
        lg.write_fits(str(tmp_path / "no_such_dir" / "x.fits"), [a])
    with pytest.raises(ValueError):
        lg.write_fits(str(tmp_path / "x.fits"), [a, np.zeros((4, 5), np.float32)])
    assert not os.path.exists(tmp_path / "x.fits")


def test_oracle_dump_layers():
    image = np.array([[1.0, 2.0], [3.0, 4.0]], np.float32)
    weight = np.array([[1.0, 0.0], [0.25, 2.0]], np.float32)
    model = np.array([[1.0, 5.0], [1.0, 3.0]], np.float32)
    raw = np.array([[2.0, 4.0], [0.0, 1.0]], np.float32)
    error = np.array([[0.5, 1.0], [0.0, 0.25]], np.float32)
    L = dump_layers(image, weight, model, raw, error)
    assert list(L) == list(DUMP_NAMES)
    assert np.array_equal(L["RES"], image - model)
    assert L["ERR"][0, 0] == 0.25 and np.isnan(L["ERR"][1, 0]) and L["ERR"][1, 1] == 0.25
    chi2 = np.array([[0.0, 0.0], [1.0, 2.0]])
    want = np.array([[math.erfc(math.sqrt(0.5 * c)) for c in row] for row in chi2], np.float32)
    assert np.array_equal(L["PVL"], want)
    assert L["PVL"][0, 1] == 1.0  # masked pixel: chi2 = 0
