"""Model bundle files: named typed arrays in one binary file.

A bundle holds everything the hot path reads -- the parameter-independent
model (``beep_model_desc`` fields), the tables ``State::set_param`` produced for
one or more parameter sets (``g<k>.<table>``), and optionally outputs.

Layout: magic ``BEEPBND1`` then records of
``u32 name_len, name, u8 type ('d' f64 | 'i' i32), u32 ndim, u64 dims[ndim], data``.
"""
from __future__ import annotations

import struct
from typing import Dict

import numpy as np

MAGIC = b"BEEPBND1"
_DT = {b"d": np.float64, b"i": np.int32}


def read_bundle(path: str) -> Dict[str, np.ndarray]:
    out: Dict[str, np.ndarray] = {}
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:8] != MAGIC:
        raise ValueError(f"{path}: not a model bundle")
    pos = 8
    while pos < len(buf):
        (nl,) = struct.unpack_from("<I", buf, pos); pos += 4
        name = buf[pos:pos + nl].decode(); pos += nl
        t = buf[pos:pos + 1]; pos += 1
        (nd,) = struct.unpack_from("<I", buf, pos); pos += 4
        dims = struct.unpack_from("<" + "Q" * nd, buf, pos); pos += 8 * nd
        dt = np.dtype(_DT[t])
        n = int(np.prod(dims)) if nd else 1
        arr = np.frombuffer(buf, dtype=dt, count=n, offset=pos).copy().reshape(dims)
        pos += n * dt.itemsize
        out[name] = arr
    return out


def write_bundle(path: str, arrays: Dict[str, np.ndarray]) -> None:
    with open(path, "wb") as f:
        f.write(MAGIC)
        for name, a in arrays.items():
            a = np.asarray(a)
            if a.dtype.kind == "f":
                t, a = b"d", np.ascontiguousarray(a, np.float64)
            elif a.dtype.kind in "iub":
                t, a = b"i", np.ascontiguousarray(a, np.int32)
            else:
                raise TypeError(f"{name}: unsupported dtype {a.dtype}")
            nb = name.encode()
            f.write(struct.pack("<I", len(nb)) + nb + t + struct.pack("<I", a.ndim))
            f.write(struct.pack("<" + "Q" * a.ndim, *a.shape))
            f.write(a.tobytes())
