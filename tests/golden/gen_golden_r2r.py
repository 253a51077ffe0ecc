"""Generate the r2r golden fixtures from the reference FFTW itself.

Run in a checkout where the reference sources exist (compiled by
``make -C oracle ref`` into ``oracle/_ref/``, codelet-free):

    python tests/golden/gen_golden_r2r.py

Writes ``tests/golden/golden_r2r.npz``: for each case the seeded input and
the reference's r2r output from its own r2r planner (``fftw_plan_many_r2r``)
in double and in long double (stored as a float64 hi + float32 lo pair, as
in gen_golden.py).  The codelet-free build plans odd lengths of every kind
except REDFT00 and RODFT00 (whose logical sizes are even), so the cases are
odd lengths of those nine kinds; inputs are numpy PCG64 draws with the seed
recorded per case.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.oracle import Reference, build  # noqa: E402

KINDS = [0, 1, 2, 4, 5, 6, 8, 9, 10]      # fftw_r2r_kind values the codelet-free build plans at odd n
SIZES = [1, 3, 5, 9, 15, 21, 105]
HOWMANY = 2


def split_dd(a):
    hi = a.astype(np.float64)
    lo = (a - hi.astype(a.dtype)).astype(np.float64)
    return hi, lo


def main():
    build(ref=True)
    refd, refl = Reference("d"), Reference("l")
    out, meta = {}, []
    i = 0
    for kind in KINDS:
        for n in SIZES:
            seed = 5000 + i
            x = np.random.default_rng(seed).standard_normal(HOWMANY * n)
            yd = refd.r2r(x, n, kind)
            yl = refl.r2r(x.astype(np.longdouble), n, kind)
            assert yd is not None and yl is not None, (kind, n)
            key = f"r2r{i:03d}"
            hi, lo = split_dd(yl)
            out[key + "_x"] = x
            out[key + "_yd"] = yd
            out[key + "_yl_hi"] = hi
            out[key + "_yl_lo"] = lo.astype(np.float32)
            meta.append({"key": key, "kind": kind, "n": n, "howmany": HOWMANY, "seed": seed})
            i += 1
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "golden_r2r.npz"), **out)
    print(f"wrote {len(meta)} cases")


if __name__ == "__main__":
    main()
