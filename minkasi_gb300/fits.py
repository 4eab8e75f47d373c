"""Minimal FITS image I/O for maps (astropy is not a dependency).

SkyMap.write / PolMap.write in the reference (minkasi/maps/skymap.py:705-722,
minkasi/maps/polmap.py:585-622) write a primary HDU holding the transposed
map with the header of the map's CAR WCS (astropy's WCS.to_header()).  This
module writes the same image: a primary HDU (FITS 4.0: 2880-byte blocks of
80-character ASCII cards, big-endian IEEE data) with BITPIX = -64 and the
linear CAR WCS keywords, and reads such files back.  It covers the single
image HDUs that map files are; anything else is out of its scope.
"""
from __future__ import annotations

import math
import os
from typing import Dict, List, Sequence, Tuple

import numpy as np

BLOCK = 2880


def _card(key: str, value, comment: str = "") -> str:
    if isinstance(value, bool):
        v = ("T" if value else "F").rjust(20)
    elif isinstance(value, (int, np.integer)):
        v = str(int(value)).rjust(20)
    elif isinstance(value, (float, np.floating)):
        x = float(value)
        if not math.isfinite(x):
            raise ValueError(f"FITS card {key}: non-finite value")
        v = repr(x).upper()
        mant, _, exp = v.partition("E")
        if "." not in mant:
            mant += ".0"
        v = (mant + ("E" + exp if exp else "")).rjust(20)
    else:
        s = str(value).replace("'", "''")
        v = ("'" + s.ljust(8) + "'").ljust(20)
    card = f"{key:<8}= {v}"
    if comment:
        card += " / " + comment
    if len(card) > 80:
        raise ValueError(f"FITS card too long: {card!r}")
    return card.ljust(80)


def car_header(wcs6: Sequence[float]) -> List[Tuple[str, object, str]]:
    """WCS keywords of a CAR projection given (crval1, crval2, crpix1, crpix2,
    cdelt1, cdelt2) in degrees, with the default pole of the projection."""
    crval1, crval2, crpix1, crpix2, cdelt1, cdelt2 = (float(v) for v in wcs6)
    return [("WCSAXES", 2, "two celestial axes"),
            ("CRPIX1", crpix1, "reference pixel, axis 1"),
            ("CRPIX2", crpix2, "reference pixel, axis 2"),
            ("CDELT1", cdelt1, "deg per pixel, axis 1"),
            ("CDELT2", cdelt2, "deg per pixel, axis 2"),
            ("CUNIT1", "deg", "unit of axis 1"),
            ("CUNIT2", "deg", "unit of axis 2"),
            ("CTYPE1", "RA---CAR", "RA, CAR projection"),
            ("CTYPE2", "DEC--CAR", "Dec, CAR projection"),
            ("CRVAL1", crval1, "deg at the reference pixel, axis 1"),
            ("CRVAL2", crval2, "deg at the reference pixel, axis 2"),
            ("LONPOLE", 0.0 if crval2 >= 0 else 180.0, "native longitude of the celestial pole"),
            ("LATPOLE", 90.0, "native latitude of the celestial pole"),
            ("RADESYS", "ICRS", "reference frame")]


def write_image(fname: str, data: np.ndarray, cards: Sequence[Tuple[str, object, str]] = (),
                overwrite: bool = True) -> None:
    """A primary HDU with ``data`` (C order: the last axis is NAXIS1) as FP64."""
    data = np.ascontiguousarray(data, dtype=">f8")
    fname = os.path.abspath(fname)
    if os.path.exists(fname) and not overwrite:
        raise FileExistsError(fname)
    os.makedirs(os.path.dirname(fname), exist_ok=True)
    head = [_card("SIMPLE", True, "conforms to FITS standard"),
            _card("BITPIX", -64, "array data type"),
            _card("NAXIS", data.ndim, "number of array dimensions")]
    for i, n in enumerate(reversed(data.shape)):
        head.append(_card(f"NAXIS{i + 1}", int(n)))
    head += [_card(k, v, c) for k, v, c in cards]
    head.append("END".ljust(80))
    text = "".join(head)
    text += " " * (-len(text) % BLOCK)
    raw = data.tobytes()
    with open(fname, "wb") as f:
        f.write(text.encode("ascii"))
        f.write(raw)
        f.write(b"\0" * (-len(raw) % BLOCK))


def _value(s: str):
    s = s.strip()
    if s.startswith("'"):
        end = s.rfind("'")
        return s[1:end].replace("''", "'").rstrip()
    if "/" in s:
        s = s.split("/", 1)[0].strip()
    if s in ("T", "F"):
        return s == "T"
    try:
        return int(s)
    except ValueError:
        return float(s.replace("D", "E"))


def read_image(fname: str) -> Tuple[np.ndarray, Dict[str, object]]:
    """The data and header keywords of a file's primary HDU."""
    with open(fname, "rb") as f:
        hdr: Dict[str, object] = {}
        done = False
        while not done:
            block = f.read(BLOCK)
            if len(block) < BLOCK:
                raise ValueError(f"{fname}: truncated FITS header")
            for i in range(0, BLOCK, 80):
                card = block[i:i + 80].decode("ascii")
                key = card[:8].strip()
                if key == "END":
                    done = True
                    break
                if card[8:10] == "= ":
                    hdr[key] = _value(card[10:])
        bitpix = int(hdr["BITPIX"])
        dtypes = {-64: ">f8", -32: ">f4", 8: "u1", 16: ">i2", 32: ">i4", 64: ">i8"}
        shape = tuple(int(hdr[f"NAXIS{i}"]) for i in range(int(hdr["NAXIS"]), 0, -1))
        count = int(np.prod(shape)) if shape else 0
        data = np.frombuffer(f.read(count * abs(bitpix) // 8), dtype=dtypes[bitpix]).reshape(shape)
    return data.astype(np.float64 if bitpix < 0 else data.dtype.newbyteorder("=")), hdr
