"""Minimal FITS image reader (numpy only).

Lensed reads its image, weight, mask and PSF through CFITSIO
(src/data.c:54-370).  CFITSIO is not a dependency here; this reader covers
what the likelihood path needs:

* primary or IMAGE extension HDUs, 2-D, BITPIX 8/16/32/64/-32/-64, big-endian,
  with BSCALE/BZERO applied;
* "first HDU that holds an image" selection, as CFITSIO's image opening does
  for files whose primary HDU is empty (Lensed 1.2+ output files);
* an optional extended-filename section ``file.fits[x0:x1,y0:y1]`` giving the
  pixel coordinate system (src/data.c:236-278): origin (x0, y0) and a step of
  +1 or -1 per axis.

Arrays are returned C-ordered as (height, width) with row 0 the bottom row of
the image (FITS order), so ``a.ravel()`` is the pixel index k = x + W*y used
by the render kernel.
"""
from __future__ import annotations

import re
from dataclasses import dataclass
from typing import List, Optional, Tuple

import numpy as np

__all__ = ["HDU", "read_hdus", "read_image", "parse_section"]

_BLOCK = 2880
_DTYPES = {8: ">u1", 16: ">i2", 32: ">i4", 64: ">i8", -32: ">f4", -64: ">f8"}


@dataclass
class HDU:
    header: dict
    data: Optional[np.ndarray]

    @property
    def name(self) -> str:
        return str(self.header.get("EXTNAME", "")).strip()


def _parse_value(v: str):
    v = v.strip()
    if v.startswith("'"):
        end = v.find("'", 1)
        while end != -1 and end + 1 < len(v) and v[end + 1] == "'":
            end = v.find("'", end + 2)
        return v[1:end].replace("''", "'").rstrip()
    v = v.split("/")[0].strip()
    if v in ("T", "F"):
        return v == "T"
    try:
        return int(v)
    except ValueError:
        pass
    try:
        return float(v.replace("D", "E"))
    except ValueError:
        return v


def read_hdus(path: str) -> List[HDU]:
    raw = open(path, "rb").read()
    off = 0
    hdus: List[HDU] = []
    while off + _BLOCK <= len(raw):
        header: dict = {}
        done = False
        while not done:
            if off + _BLOCK > len(raw):
                raise ValueError(f"{path}: truncated header")
            block = raw[off : off + _BLOCK]
            off += _BLOCK
            for i in range(36):
                card = block[i * 80 : (i + 1) * 80].decode("ascii", "replace")
                key = card[:8].strip()
                if key == "END":
                    done = True
                    break
                if card[8:10] == "= " and key not in header:
                    header[key] = _parse_value(card[10:])
        bitpix = int(header.get("BITPIX", 8))
        naxis = int(header.get("NAXIS", 0))
        shape = [int(header[f"NAXIS{i + 1}"]) for i in range(naxis)]
        n = int(np.prod(shape)) if naxis > 0 else 0
        nbytes = abs(bitpix) // 8 * n
        data = None
        if n > 0 and not header.get("XTENSION", "IMAGE").startswith("BINTABLE"):
            arr = np.frombuffer(raw, dtype=_DTYPES[bitpix], count=n, offset=off)
            arr = arr.reshape(shape[::-1]).astype(np.float64 if bitpix in (-64, 64, 32) else np.float32)
            bscale = float(header.get("BSCALE", 1.0))
            bzero = float(header.get("BZERO", 0.0))
            if bscale != 1.0 or bzero != 0.0:
                arr = arr * bscale + bzero
            data = arr
        hdus.append(HDU(header, data))
        off += (nbytes + _BLOCK - 1) // _BLOCK * _BLOCK
    return hdus


def parse_section(spec: str) -> Tuple[str, Optional[Tuple[int, int, int, int]]]:
    """Split ``file.fits[x0:x1,y0:y1]`` into the file name and the section."""
    m = re.match(r"^(.*?)\[(-?\d+):(-?\d+),(-?\d+):(-?\d+)\]$", spec.strip())
    if not m:
        return spec, None
    return m.group(1), tuple(int(m.group(i)) for i in range(2, 6))  # type: ignore[return-value]


def read_image(spec: str, hdu: Optional[int] = None, dtype=np.float32):
    """Read an image and its pixel coordinate system.

    Returns ``(array[H, W], pcs)`` with ``pcs = (rx, ry, sx, sy)``.  Without a
    section the pcs is (1, 1, 1, 1); with ``[x0:x1,y0:y1]`` the image is cut
    to the section and the pcs is (x0, y0, +-1, +-1).
    """
    path, sec = parse_section(spec)
    hdus = read_hdus(path)
    if hdu is None:
        picked = next((h for h in hdus if h.data is not None and h.data.ndim == 2), None)
    else:
        picked = hdus[hdu]
    if picked is None or picked.data is None:
        raise ValueError(f"{path}: no image HDU")
    a = picked.data
    pcs = (1.0, 1.0, 1.0, 1.0)
    if sec is not None:
        x0, x1, y0, y1 = sec
        sx = 1 if x1 >= x0 else -1
        sy = 1 if y1 >= y0 else -1
        a = a[y0 - 1 : (y1 - 1) + sy if (y1 - 1) + sy >= 0 else None : sy,
              x0 - 1 : (x1 - 1) + sx if (x1 - 1) + sx >= 0 else None : sx]
        pcs = (float(x0), float(y0), float(sx), float(sy))
    return np.ascontiguousarray(a, dtype=dtype), pcs
