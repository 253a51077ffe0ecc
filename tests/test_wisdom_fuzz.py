"""Wisdom import robustness, checked without a GPU: seeded mutations of a
valid wisdom text (deleted, inserted and replaced bytes, random bytes) never
crash the parser, a rejected import leaves the existing wisdom intact, and
the plans made under any accepted mutation keep every pass inside the launch
limits (dry-run plans)."""
import ctypes
import random

import pytest

import fftw3_gb300 as g

GOOD = (b'(fftw-3.3.10-gb300 fftwf_wisdom #x67623330304c4942\n'
        b'  (gb300-pass "c2c p4 n1024" #x0 #x2 #x0 #x0 #x0)\n'
        b'  (gb300-pass "r2c p4 n4096" #x1 #x4 #x0 #x0 #x40)\n)\n')


@pytest.fixture(autouse=True)
def dry(lib):
    g.set_dry_run(True)
    lib.fftwf_forget_wisdom()
    yield
    lib.fftwf_forget_wisdom()
    g.set_dry_run(False)


def mutate(rng, text, edits):
    s = bytearray(text)
    for _ in range(edits):
        op, i = rng.random(), rng.randrange(len(s) + 1)
        if op < 0.4 and s:
            del s[i % len(s)]
        elif op < 0.8:
            s.insert(i, rng.randrange(1, 256))
        else:
            s[i % len(s)] = rng.choice(b'()"# \n0123456789abcdefx-')
    return bytes(s)


def test_mutated_wisdom_never_crashes_and_rejections_keep_wisdom(lib):
    assert lib.fftwf_import_wisdom_from_string(GOOD) == 1
    before = ctypes.string_at(lib.fftwf_export_wisdom_to_string())
    rng = random.Random(5)
    accepted = 0
    for _ in range(3000):
        text = mutate(rng, GOOD, rng.randint(1, 8)) if rng.random() > 0.05 else \
            bytes(rng.randrange(1, 256) for _ in range(rng.randint(0, 300)))
        if lib.fftwf_import_wisdom_from_string(text):
            accepted += 1
            lib.fftwf_forget_wisdom()
            assert lib.fftwf_import_wisdom_from_string(GOOD) == 1
        else:
            assert ctypes.string_at(lib.fftwf_export_wisdom_to_string()) == before
    assert accepted < 3000


def test_plans_under_accepted_mutations_stay_in_limits(lib):
    rng = random.Random(6)
    checked = 0
    for _ in range(3000):
        text = bytearray(GOOD)
        for _ in range(rng.randint(1, 4)):
            text[rng.randrange(len(text))] = rng.choice(b"0123456789abcdefx")
        lib.fftwf_forget_wisdom()
        if not lib.fftwf_import_wisdom_from_string(bytes(text)):
            continue
        for make in (lambda: g.plan_many_dft([1024], 64, 1 << 20, 1 << 30, prec="f"),
                     lambda: g.plan_many_dft_r2c([4096], 64, 1 << 20, 1 << 30, prec="f")):
            try:
                p = make()
            except RuntimeError:
                continue
            checked += 1
            for ps in p.passes():
                assert 1 <= ps["threads"] <= 1024 and ps["tb"] >= 1 and 0 <= ps["smem"] <= 232448
                assert ps["blocks"] >= 1
    assert checked > 100
