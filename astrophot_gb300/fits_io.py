"""Minimal FITS image I/O (FITS Standard 4.0: 2880-byte blocks, 80-character header cards,
big-endian data; the CONTINUE long-string convention).  It reads and writes the image HDU lists
the reference's ``Image.save`` / ``Image.load`` produce through astropy
(``astrophot/image/image_object.py:409-428``): a primary HDU and IMAGE extensions, each with
string-valued header keys.  Only image HDUs are written; other extension types are skipped on
reading.
"""

from __future__ import annotations

import math
from typing import Dict, List, Tuple

import numpy as np

BLOCK = 2880
CARD = 80

_BITPIX = {np.dtype(np.uint8): 8, np.dtype(np.int16): 16, np.dtype(np.int32): 32, np.dtype(np.int64): 64,
           np.dtype(np.float32): -32, np.dtype(np.float64): -64}
_DTYPE = {8: ">u1", 16: ">i2", 32: ">i4", 64: ">i8", -32: ">f4", -64: ">f8"}


# -- writing ----------------------------------------------------------------------------------

def _fmt_value(v) -> str:
    if isinstance(v, (bool, np.bool_)):
        return f"{'T' if v else 'F':>20}"
    if isinstance(v, (int, np.integer)):
        return f"{int(v):>20d}"
    if isinstance(v, (float, np.floating)):
        s = repr(float(v)).upper()
        if "E" not in s and "." not in s and s not in ("NAN", "INF", "-INF"):
            s += "."
        return f"{s:>20}"
    raise TypeError(type(v))


def _cards(key: str, value) -> List[str]:
    key = key.upper()
    if len(key) > 8:
        raise ValueError(f"FITS keywords have at most 8 characters: {key}")
    if not isinstance(value, str):
        return [f"{key:<8}= {_fmt_value(value)}".ljust(CARD)]
    s = value.replace("'", "''")
    if len(s) <= 68:
        return [f"{key:<8}= '{s:<8}'".ljust(CARD)]
    # long string: pieces ending in '&' continued on CONTINUE cards (at most 67 characters each,
    # never splitting an escaped quote)
    out, first = [], True
    while s:
        n = 67
        piece = s[:n]
        if piece.endswith("'") and not piece.endswith("''") and len(s) > n:
            piece = piece[:-1]
        s = s[len(piece):]
        text = piece + ("&" if s else "")
        out.append((f"{key:<8}= '{text}'" if first else f"CONTINUE  '{text}'").ljust(CARD))
        first = False
    return out


def _header_bytes(cards: List[str]) -> bytes:
    text = "".join(cards) + "END".ljust(CARD)
    text += " " * ((-len(text)) % BLOCK)
    return text.encode("ascii")


def _data_bytes(data: np.ndarray) -> bytes:
    raw = np.ascontiguousarray(data).astype(_DTYPE[_BITPIX[data.dtype]], copy=False).tobytes()
    return raw + b"\0" * ((-len(raw)) % BLOCK)


def write_hdus(filename: str, hdus: List[Tuple[np.ndarray, Dict[str, object]]]):
    """Write [(data, header keys), ...]: the first as the primary HDU, the rest as IMAGE
    extensions.  Booleans are stored as int64, other types as they are (float64, int...)."""
    with open(filename, "wb") as f:
        for k, (data, header) in enumerate(hdus):
            data = np.asarray(data)
            if data.dtype == np.bool_:
                data = data.astype(np.int64)
            if data.dtype not in _BITPIX:
                data = data.astype(np.float64)
            cards = _cards("SIMPLE", True) if k == 0 else _cards("XTENSION", "IMAGE")
            cards += _cards("BITPIX", _BITPIX[data.dtype])
            cards += _cards("NAXIS", data.ndim)
            for i, n in enumerate(reversed(data.shape)):
                cards += _cards(f"NAXIS{i + 1}", int(n))
            if k == 0:
                cards += _cards("EXTEND", True)
            else:
                cards += _cards("PCOUNT", 0) + _cards("GCOUNT", 1)
            for key, value in header.items():
                cards += _cards(key, value)
            f.write(_header_bytes(cards))
            f.write(_data_bytes(data))


# -- reading ----------------------------------------------------------------------------------

def _parse_value(text: str):
    t = text.strip()
    if t.startswith("'"):
        out, i = [], 1
        while i < len(t):
            if t[i] == "'":
                if i + 1 < len(t) and t[i + 1] == "'":
                    out.append("'")
                    i += 2
                    continue
                break
            out.append(t[i])
            i += 1
        return "".join(out).rstrip()
    t = t.split("/")[0].strip()
    if t == "T":
        return True
    if t == "F":
        return False
    if t == "":
        return None
    try:
        return int(t)
    except ValueError:
        return float(t.replace("D", "E"))


def _read_header(f) -> Dict[str, object]:
    header: Dict[str, object] = {}
    last = None
    while True:
        block = f.read(BLOCK)
        if len(block) < BLOCK:
            raise ValueError("truncated FITS header")
        for j in range(0, BLOCK, CARD):
            card = block[j : j + CARD].decode("ascii")
            key = card[:8].strip()
            if key == "END":
                return header
            if key == "CONTINUE" and last is not None and isinstance(header[last], str):
                prev = header[last]
                if prev.endswith("&"):
                    header[last] = prev[:-1] + _parse_value(card[8:])
                continue
            if card[8:10] == "= ":
                header[key] = _parse_value(card[10:])
                last = key


def read_hdus(filename: str) -> List[Tuple[np.ndarray, Dict[str, object]]]:
    """[(data, header dict), ...] of every image HDU of the file (BSCALE / BZERO applied)."""
    out = []
    with open(filename, "rb") as f:
        while True:
            start = f.read(1)
            if not start:
                break
            f.seek(-1, 1)
            h = _read_header(f)
            bitpix, naxis = int(h["BITPIX"]), int(h.get("NAXIS", 0))
            shape = [int(h[f"NAXIS{i + 1}"]) for i in range(naxis)]
            n = math.prod(shape) if naxis else 0
            pcount, gcount = int(h.get("PCOUNT", 0)), int(h.get("GCOUNT", 1))
            nbytes = abs(bitpix) // 8 * gcount * (pcount + n)
            raw = f.read(nbytes)
            f.read((-nbytes) % BLOCK)
            if "XTENSION" in h and str(h["XTENSION"]).strip() != "IMAGE":
                continue
            data = np.frombuffer(raw[: abs(bitpix) // 8 * n], dtype=_DTYPE[bitpix]).reshape(shape[::-1]) if n else None
            if data is not None:
                data = data.astype(data.dtype.newbyteorder("="))
                if "BSCALE" in h or "BZERO" in h:
                    data = data * float(h.get("BSCALE", 1.0)) + float(h.get("BZERO", 0.0))
            out.append((data, h))
    return out
