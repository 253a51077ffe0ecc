"""Generate the golden fixtures from the reference FFTW itself.

Run in a checkout where the reference sources exist (they are compiled by
``make -C oracle ref`` into ``oracle/_ref/``, codelet-free):

    python tests/golden/gen_golden.py

Writes ``tests/golden/golden.npz``.  Each case stores the seeded input and
the reference's output computed in double (``fftw_``) and in long double
(``fftwl_``).  Long-double outputs are stored as a pair of float64 arrays
(hi as float64 + lo as float32, a double-double split) so the file reads the same on x86-64
(80-bit long double) and aarch64 (binary128).

The reference publishes no stored golden outputs of its own (its tests are
property checks, libbench2/verify-lib.c:260-434), so these fixtures are
outputs of the reference run here, on inputs drawn from numpy's PCG64 with
the seed recorded per case.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.oracle import Reference, build  # noqa: E402

# (kind, shape, howmany, sign) -- sizes the reference finishes instantly.
CASES = [
    ("c2c", [1], 3, -1), ("c2c", [2], 2, -1), ("c2c", [3], 2, 1), ("c2c", [4], 2, -1),
    ("c2c", [5], 2, -1), ("c2c", [7], 1, 1), ("c2c", [8], 2, -1), ("c2c", [16], 2, 1),
    ("c2c", [17], 2, -1), ("c2c", [32], 2, -1), ("c2c", [60], 2, -1), ("c2c", [64], 2, 1),
    ("c2c", [173], 1, -1), ("c2c", [256], 2, -1), ("c2c", [1021], 1, -1), ("c2c", [1024], 2, -1),
    ("c2c", [1024], 2, 1), ("c2c", [2048], 1, -1), ("c2c", [4096], 2, -1), ("c2c", [4096], 1, 1),
    ("c2c", [8192], 1, -1), ("c2c", [210], 2, -1), ("c2c", [1000], 1, 1), ("c2c", [4093], 1, -1),
    ("c2c", [8, 12], 2, -1), ("c2c", [16, 16], 1, 1), ("c2c", [4, 6, 10], 1, -1),
    ("c2c", [8, 8, 8], 1, -1), ("c2c", [32, 64], 1, -1),
    ("r2c", [15], 2, -1), ("r2c", [16], 2, -1), ("r2c", [1024], 2, -1), ("r2c", [4096], 1, -1),
    ("r2c", [8, 6], 2, -1), ("r2c", [64, 64], 1, -1), ("r2c", [6, 10, 14], 1, -1),
    ("c2r", [15], 2, 1), ("c2r", [16], 2, 1), ("c2r", [1024], 2, 1), ("c2r", [4096], 1, 1),
    ("c2r", [8, 6], 2, 1), ("c2r", [64, 64], 1, 1),
]


def split_dd(a):
    """long double -> (hi, lo) float64 pair."""
    hi = a.astype(np.float64)
    lo = (a - hi.astype(a.dtype)).astype(np.float64)
    return hi, lo


def main():
    build(ref=True)
    refd, refl = Reference("d"), Reference("l")
    out = {}
    meta = []
    for i, (kind, shape, hm, sign) in enumerate(CASES):
        seed = 1000 + i
        rng = np.random.default_rng(seed)
        tot = int(np.prod(shape))
        nc = tot // shape[-1] * (shape[-1] // 2 + 1)
        if kind == "c2c":
            x = rng.standard_normal(hm * tot) + 1j * rng.standard_normal(hm * tot)
            yd = refd.c2c(x, shape, sign)
            yl = refl.c2c(x.astype(np.clongdouble), shape, sign)
        elif kind == "r2c":
            x = rng.standard_normal(hm * tot)
            yd = refd.r2c(x, shape)
            yl = refl.r2c(x.astype(np.longdouble), shape)
        else:
            x = rng.standard_normal(hm * nc) + 1j * rng.standard_normal(hm * nc)
            yd = refd.c2r(x, shape)
            yl = refl.c2r(x.astype(np.clongdouble), shape)
        key = f"case{i:03d}"
        out[key + "_x"] = x
        out[key + "_yd"] = yd
        if np.iscomplexobj(yl):
            hr, lr = split_dd(yl.real)
            hi_, li = split_dd(yl.imag)
            out[key + "_yl_hi"] = hr + 1j * hi_
            out[key + "_yl_lo"] = (lr + 1j * li).astype(np.complex64)
        else:
            h, l_ = split_dd(yl)
            out[key + "_yl_hi"] = h
            out[key + "_yl_lo"] = l_.astype(np.float32)
        meta.append({"key": key, "kind": kind, "shape": shape, "howmany": hm, "sign": sign, "seed": seed})
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print(f"wrote {len(meta)} cases")


if __name__ == "__main__":
    main()
