"""bench.py's contract, checked without a GPU: the metric arithmetic
(5 N log2 N per complex transform, 2.5 N log2 N per real or r2r transform,
one read plus one write of the arrays) for the named workloads, and the
reference arm's JSON line (it times the host-side implementation, so it
runs here) with every key the contract asks for."""
import argparse
import contextlib
import io
import json
import math

import bench


def test_flops_and_bytes_per_step():
    # fftwf c2c 4096 x 65536: 5 * 4096 * 12 * 65536 flops, 2 GiB in + 2 GiB out
    assert bench.flops_per_step("c2c", [4096], 65536) == 5 * 4096 * 12 * 65536
    assert bench.bytes_per_step("c2c", [4096], 65536, "f") == 2 * 4096 * 8 * 65536
    # r2c 16384 x 16384: half the complex count; 16384 reals in, 8193 complex out
    assert bench.flops_per_step("r2c", [16384], 16384) == 2.5 * 16384 * 14 * 16384
    assert bench.bytes_per_step("r2c", [16384], 16384, "f") == (16384 * 4 + 8193 * 8) * 16384
    # 2D r2c 8192^2 and 3D c2c 512^3 (log2 of the whole size, as the reference's mflops)
    assert bench.bytes_per_step("r2c", [8192, 8192], 1, "f") == 8192 * (8192 * 4 + 4097 * 8)
    assert math.isclose(bench.flops_per_step("c2c", [512, 512, 512], 1), 5 * 2 ** 27 * 27)
    # r2r: 2.5 N log2 N (libbench2/mflops.c), reals in and out
    assert bench.flops_per_step("r2r", [4096], 65536) == 2.5 * 4096 * 12 * 65536
    assert bench.bytes_per_step("r2r", [4096], 65536, "f") == 2 * 4096 * 4 * 65536
    # double c2c 1024 x 4096
    assert bench.bytes_per_step("c2c", [1024], 4096, "d") == 2 * 1024 * 16 * 4096


def test_uneven_lengths_are_seeded_and_in_range():
    import numpy as np
    a = bench.uneven_lengths(np.random.default_rng(2024), 500)
    b = bench.uneven_lengths(np.random.default_rng(2024), 500)
    assert a == b and all(2 <= n <= 65536 for n in a)


def test_reference_arm_json_line(lib):
    args = argparse.Namespace(gpus=1, steps=1, warmup=0, impl="reference", workload="c2c4096", howmany=0,
                              no_e2e=False, no_cpu=False, no_tc=False)
    out = io.StringIO()
    with contextlib.redirect_stdout(out):
        bench.run_reference_arm(args)
    line = json.loads(out.getvalue().strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "impl", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["unit"] == "Gflop/s" and line["value"] > 0
    assert line["metric"] == bench.METRIC and line["higher_is_better"] is True
    assert line["e2e"] == {"value": line["value"], "unit": "Gflop/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["cpu_baseline"]["kind"] in ("reference", "port") and line["cpu_baseline"]["cores"] >= 1
    assert line["config"]["workload"].startswith("c2c4096")
