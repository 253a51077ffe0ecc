"""Plan-set host logic without a GPU (sets planned in dry run): how uneven
lengths become work-queue items — singles grouped by length, Bluestein and
Rader singles for primes, column and row tiles of the two-pass long lengths —
the item order the queue's bounded waits rely on, the tile widths, the item
body choice, and the shared-memory budget of three small-tile CTAs per SM."""
import ctypes

import numpy as np
import pytest

import fftw3_gb300 as g

GB_KIND_C2C, GB_KIND_BLUESTEIN, GB_KIND_RADER = 0, 3, 5
GB_VAR_REG, GB_VAR_GEN = 0, 1
# complex elements of one small-tile buffer: 16 (float) or 8 (double)
# transforms of 256 points in the padded layout (n + n/16 + 1 apart)
QBUF = {"f": 16 * 273, "d": 8 * 273}


def gen_sms(n):
    return n + n // 16 + 1


@pytest.fixture(autouse=True)
def dry(lib):
    g.set_dry_run(True)
    yield
    g.set_dry_run(False)


def _plan_set(lengths, prec="f", flags=None):
    lib = g.load()
    pfx = "fftwf_" if prec == "f" else "fftw_"
    plans = [g.plan_many_dft([int(n)], 1, 1 << 20, 1 << 30, -1, g.FFTW_ESTIMATE, prec) for n in lengths]
    arr = (ctypes.c_void_p * len(plans))(*[p.ptr for p in plans])
    f = getattr(lib, pfx + "gb300_plan_set")
    f.restype = ctypes.c_void_p
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_uint]
    s = f(len(plans), arr, g.FFTW_ESTIMATE if flags is None else flags)
    return lib, pfx, s, plans


def _info(lib, pfx, s):
    v = [ctypes.c_int() for _ in range(5)]
    fn = getattr(lib, pfx + "gb300_set_info")
    fn.argtypes = [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_int)] * 5
    assert fn(s, *[ctypes.byref(x) for x in v]) == 0
    return dict(zip(["nitems", "ntransforms", "nlong", "grid", "smem"], [x.value for x in v]))


def _items(lib, pfx, s, n):
    fn = getattr(lib, pfx + "gb300_set_item_info")
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.POINTER(ctypes.c_int)] * 6
    out = []
    for i in range(n):
        v = [ctypes.c_int() for _ in range(6)]
        assert fn(s, i, *[ctypes.byref(x) for x in v]) == 0
        out.append(dict(zip(["kind", "nfft", "tb", "variant", "queue", "role"], [x.value for x in v])))
    return out


def _destroy(lib, pfx, s):
    fn = getattr(lib, pfx + "gb300_destroy_set")
    fn.argtypes = [ctypes.c_void_p]
    fn(s)


def _smooth(n):
    for p in (2, 3, 5, 7, 11, 13):
        while n % p == 0:
            n //= p
    return n == 1


def test_uneven10k_items_and_order():
    """The 10,000-plan uneven workload: every transform placed, one two-pass
    long transform per 13-smooth length above 4096; in the small-tile queue
    every column tile comes before every single and every row tile after
    them (a claimed item never waits on a later one); tiles of long lengths
    fit one small-tile buffer, 16 columns wide for most (factors of at most
    256 points); singles hold at most 32 transforms and fit one buffer."""
    import bench
    lengths = bench.uneven_lengths(np.random.default_rng(2024), 10000)
    lib, pfx, s, plans = _plan_set(lengths)
    assert s, g.last_error()
    info = _info(lib, pfx, s)
    assert info["ntransforms"] == 10000
    assert info["nlong"] == sum(1 for n in lengths if n > 4096 and _smooth(n))
    items = _items(lib, pfx, s, info["nitems"])
    small = [it for it in items if it["queue"] == 0]
    large = [it for it in items if it["queue"] == 1]
    roles = [it["role"] for it in small]
    first_single = roles.index(0)
    first_row = roles.index(2)
    assert all(r == 1 for r in roles[:first_single])
    assert all(r == 0 for r in roles[first_single:first_row])
    assert all(r == 2 for r in roles[first_row:])
    assert sum(1 for r in roles if r == 1) > 0 and sum(1 for r in roles if r == 2) > 0
    tiles = [it for it in small if it["role"]]
    for it in tiles:
        assert it["kind"] == GB_KIND_C2C and it["tb"] in (1, 2, 4, 8, 16)
        assert it["tb"] * gen_sms(it["nfft"]) <= QBUF["f"]
    # the factors of most long lengths are at most 256 points: 16-column tiles
    assert sum(1 for it in tiles if it["tb"] == 16) >= 0.9 * len(tiles)
    for it in small:
        if not it["role"]:
            assert 1 <= it["tb"] <= 32 and it["tb"] * gen_sms(it["nfft"]) <= QBUF["f"]
    # large tiles: primes whose Bluestein convolution needs 8192 points
    assert large and all(it["kind"] == GB_KIND_BLUESTEIN and it["nfft"] == 8192 and it["role"] == 0 for it in large)
    _destroy(lib, pfx, s)


@pytest.mark.parametrize("prec", ["f", "d"])
def test_small_tile_budget(prec):
    """The largest small-tile item fits two buffers of QBUF elements, so three
    256-thread CTAs (each with up to 2 KB of static shared memory and the
    1 KB the system reserves) share an SM's 228 KB."""
    lengths = [64, 256, 1000, 2048, 4096, 8192, 65536, 60000, 97, 4093] if prec == "f" else \
              [64, 256, 1000, 2048, 4096, 16384, 97, 2039]
    lib, pfx, s, plans = _plan_set(lengths, prec)
    assert s, g.last_error()
    info = _info(lib, pfx, s)
    cs = 8 if prec == "f" else 16
    assert info["smem"] <= 2 * QBUF[prec] * cs
    assert 3 * (info["smem"] + 2048 + 1024) <= 233472
    assert info["grid"] == 0   # dry run: no launch shape
    _destroy(lib, pfx, s)


def test_item_body_choice(monkeypatch):
    """Power-of-two float items of 64..4096 points run the runtime-radix body
    unless wisdom or FFTW_GB300_QUEUE_BODY=reg asks for the register stages;
    other lengths always run the runtime-radix body."""
    lengths = [64, 128, 512, 4096, 60, 1000, 97]
    for body, want in ((None, GB_VAR_GEN), ("reg", GB_VAR_REG), ("gen", GB_VAR_GEN)):
        if body is None:
            monkeypatch.delenv("FFTW_GB300_QUEUE_BODY", raising=False)
        else:
            monkeypatch.setenv("FFTW_GB300_QUEUE_BODY", body)
        lib, pfx, s, plans = _plan_set(lengths)
        items = _items(lib, pfx, s, _info(lib, pfx, s)["nitems"])
        for it in items:
            pow2 = it["kind"] == GB_KIND_C2C and it["nfft"] & (it["nfft"] - 1) == 0 and 64 <= it["nfft"] <= 4096
            assert it["variant"] == (want if pow2 else GB_VAR_GEN), it
        _destroy(lib, pfx, s)


def test_rader_singles(monkeypatch):
    """FFTW_GB300_PRIME=rader: primes with 13-smooth n-1 become Rader singles
    of n-1 points; the others stay Bluestein."""
    monkeypatch.setenv("FFTW_GB300_PRIME", "rader")
    lengths = [17, 97, 401, 4093, 1201]
    lib, pfx, s, plans = _plan_set(lengths)
    items = _items(lib, pfx, s, _info(lib, pfx, s)["nitems"])
    got = sorted((it["kind"], it["nfft"]) for it in items)
    want = sorted((GB_KIND_RADER, n - 1) if _smooth(n - 1) else
                  (GB_KIND_BLUESTEIN, 1 << int(np.ceil(np.log2(2 * n - 1)))) for n in lengths)
    assert got == want
    _destroy(lib, pfx, s)


def test_wisdom_only_without_wisdom_is_refused():
    lib = g.load()
    lib.fftwf_forget_wisdom()
    lib_, pfx, s, plans = _plan_set([64, 1000], flags=g.FFTW_ESTIMATE | g.FFTW_WISDOM_ONLY)
    assert not s
    assert "WISDOM_ONLY" in g.last_error()


def test_dry_run_set_does_not_execute():
    lib, pfx, s, plans = _plan_set([64, 1000])
    fn = getattr(lib, pfx + "gb300_execute_set")
    fn.argtypes = [ctypes.c_void_p]
    assert fn(s) == -1
    assert "dry run" in g.last_error()
    item = getattr(lib, pfx + "gb300_set_item_info")
    item.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.POINTER(ctypes.c_int)] * 6
    v = [ctypes.c_int() for _ in range(6)]
    assert item(s, 10 ** 6, *[ctypes.byref(x) for x in v]) == -1
    _destroy(lib, pfx, s)


def test_set_wisdom_entries_steer_items():
    """The set tuner's wisdom entries ("set p4 n<n>": variant, tb, load, store,
    n1, groups, order), imported as text, steer the items: the register body
    for a power-of-two length, Rader for a prime, another split for a long
    length, fewer transforms per item; with an entry for every length the
    set plans under FFTW_WISDOM_ONLY."""
    lib = g.load()
    lib.fftwf_forget_wisdom()
    head = ctypes.string_at(lib.fftwf_export_wisdom_to_string()).decode().rstrip().rstrip(")")
    ent = lambda n, *f: '  (gb300-pass "set p4 n%d" %s)\n' % (n, " ".join("#x%x" % (v & 0xffffffff) for v in f))
    text = head + ent(4096, 0, 0, 0, 0, 0, 0, 0) + ent(97, 5, 0, 0, 0, 0, 0, 0) + \
        ent(65536, -1, 0, 0, 0, 64, 0, 0) + ent(256, -1, 4, 0, 0, 0, 0, 0) + ")\n"
    assert lib.fftwf_import_wisdom_from_string(text.encode()) == 1, text
    lengths = [4096, 97, 65536, 256, 256, 256, 256, 256, 256]
    lib_, pfx, s, plans = _plan_set(lengths, flags=g.FFTW_ESTIMATE | g.FFTW_WISDOM_ONLY)
    assert s, g.last_error()
    items = _items(lib, pfx, s, _info(lib, pfx, s)["nitems"])
    by = {}
    for it in items:
        by.setdefault(it["nfft"], []).append(it)
    assert all(it["variant"] == GB_VAR_REG for it in by[4096])
    assert [it["kind"] for it in by[96]] == [GB_KIND_RADER]
    assert all(it["role"] for it in by[64] + by[1024]) and 64 in by and 1024 in by
    singles256 = [it for it in by[256] if not it["role"]]
    assert [it["tb"] for it in singles256] == [4, 2]
    _destroy(lib, pfx, s)
    # a length without an entry: refused under FFTW_WISDOM_ONLY
    lib_, pfx, s, plans = _plan_set(lengths + [1000], flags=g.FFTW_ESTIMATE | g.FFTW_WISDOM_ONLY)
    assert not s
    lib.fftwf_forget_wisdom()


@pytest.mark.parametrize("prec,seed", [("f", 1), ("f", 2), ("f", 3), ("d", 4), ("d", 5)])
def test_random_sets_cover_every_transform(prec, seed):
    """Seeded uneven sets in both precisions: every transform is a single
    (the singles' transforms per item add up) or one long transform; the
    small-tile queue keeps column tiles, singles, row tiles in that order;
    every item fits a small- or large-tile buffer."""
    import bench
    rng = np.random.default_rng(seed)
    if prec == "f":
        lengths = bench.uneven_lengths(rng, 600)
    else:
        lengths = bench.uneven_lengths(rng, 400, max_pow2=14, max_smooth=20000, max_prime=2047)
    lengths += [1, 2, 3]
    lib, pfx, s, plans = _plan_set(lengths, prec)
    assert s, g.last_error()
    info = _info(lib, pfx, s)
    items = _items(lib, pfx, s, info["nitems"])
    assert info["ntransforms"] == len(lengths)
    assert sum(it["tb"] for it in items if it["role"] == 0) + info["nlong"] == len(lengths)
    roles = [it["role"] for it in items if it["queue"] == 0]
    assert roles == sorted(roles, key=lambda r: (1, 0, 2).index(r))
    for it in items:
        cap = QBUF[prec] * (2 if it["queue"] else 1)
        assert it["tb"] * gen_sms(it["nfft"]) <= cap or it["tb"] == 1 and gen_sms(it["nfft"]) <= cap, it
    _destroy(lib, pfx, s)
