"""TEST INFRASTRUCTURE ONLY: a numpy restatement of the reference's PLY
import (src/utils/load.ts:14-172 with src/utils/plyreader.ts:1-77), used by
tests/ to check the library's importer, plus a small PLY writer for test
files.

The reference stores every imported value in a Float16Array
(@petamoriken/float16 3.8.7): the JavaScript double is rounded to f32, then
to f16 with ties to even -- numpy's float32 -> float16 conversion.
"""
from __future__ import annotations

import math
import struct

import numpy as np

SH_C0 = 0.28209479177387814


def write_ply(path, props: list[tuple[str, str]], rows: list[list[float]],
              fmt: str = "binary_little_endian") -> None:
    """props: [(type, name)] with type float/uchar/double; rows: values."""
    head = f"ply\nformat {fmt} 1.0\nelement vertex {len(rows)}\n"
    head += "".join(f"property {t} {n}\n" for t, n in props)
    head += "end_header\n"
    code = {"float": "f", "uchar": "B", "double": "d"}
    with open(path, "wb") as f:
        f.write(head.encode())
        for r in rows:
            f.write(b"".join(struct.pack("<" + code[t], v) for (t, _), v in zip(props, r)))


def f16(v) -> np.float32:
    return np.float32(np.float16(np.float32(v)))


def expected_planes(props: list[tuple[str, str]], rows: list[list[float]]):
    """load(): (59, n) planes in the context layout, SH degree, extent."""
    names = [n for _, n in props]
    types = dict((n, t) for t, n in props)
    n = len(rows)

    def raw(r, name):
        if name not in types:
            return None
        v = r[names.index(name)]
        if types[name] == "uchar":
            return v / 255.0                              # readRawVertex
        return float(np.float32(v))                       # getFloat32

    gauss = all(k in types for k in ("f_dc_0", "opacity", "rot_0", "scale_0"))
    rgb = all(k in types for k in ("red", "green", "blue")) and not gauss
    nrest = sum(1 for k in names if k.startswith("f_rest_"))
    per = nrest // 3
    deg = int(math.sqrt(per + 1) - 1) if gauss else 0
    P = np.zeros((59, n), np.float32)
    lo = [math.inf] * 3
    hi = [-math.inf] * 3
    for i, r in enumerate(rows):
        for k, a in enumerate("xyz"):
            v = raw(r, a)
            P[k, i] = f16(v)
            lo[k], hi[k] = min(lo[k], v), max(hi[k], v)
        if gauss:
            for k in range((deg + 1) ** 2):
                for c in range(3):
                    name = f"f_dc_{c}" if k == 0 else f"f_rest_{c * per + k - 1}"
                    P[11 + 3 * k + c, i] = f16(raw(r, name))
            P[10, i] = f16(raw(r, "opacity"))
            # halves (rot_0, rot_1, rot_2, rot_3) read as quaternion (rot_1, rot_2, rot_3, rot_0)
            P[9, i], P[6, i], P[7, i], P[8, i] = (f16(raw(r, f"rot_{k}")) for k in range(4))
            for k in range(3):
                P[3 + k, i] = f16(raw(r, f"scale_{k}"))
        else:
            if rgb:
                for c, ch in enumerate(("red", "green", "blue")):
                    r8 = raw(r, ch)
                    P[11 + c, i] = f16(((r8 if r8 is not None else 255) / 255.0 - 0.5) / SH_C0)
            P[10, i] = f16(-2.197)
            P[9, i], P[6, i], P[7, i], P[8, i] = 0.0, 0.0, 0.0, 1.0
            for k in range(3):
                P[3 + k, i] = f16(math.log(0.01))
    extent = max(hi[k] - lo[k] for k in range(3))
    return P, deg, extent
