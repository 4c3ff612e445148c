"""The bench's JSON line (the committed latest full line under profiles/)
against the output contract bench.py promises: the keys and their nesting,
value = 64 applies per step / ms_per_step, the roofline fraction = achieved /
peak, the end-to-end object's byte counts for a 64-ket ComplexF64 step of
the 14-spin chain, the CPU baseline's description, the clock record, and the
sub-objects for the other arithmetic forms, the batched and the served runs.
No GPU: the line is read from the file."""
import json
import os

import pytest

LINE = os.path.join(os.path.dirname(__file__), "..", "profiles", "bench_heisenberg14_batch64_line.json")


@pytest.fixture(scope="module")
def line():
    with open(LINE) as f:
        return json.loads(f.read().strip().splitlines()[-1])


def test_top_level_keys(line):
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "roofline", "cpu_baseline", "e2e", "clocks", "gpu_launches"):
        assert k in line, k
    assert line["n_gpus"] == 1 and line["higher_is_better"] is True and line["scaling"] == "weak"
    assert line["warmup"] >= 3 and line["steps"] >= 1
    assert line["vs_baseline"] is None  # no published number for this metric
    assert line["dtype"] == "c128" and line["data"].startswith("synthetic")
    assert line["config"]["workload"] == "heisenberg14_lazysum_ket_batch64"
    assert line["config"]["dim"] == 16384 and line["config"]["batch_kets"] == 64


def test_value_matches_step_time(line):
    assert line["value"] == pytest.approx(line["config"]["batch_kets"] / (line["ms_per_step"] * 1e-3), rel=1e-6)
    assert line["gpu_launches"] >= line["steps"]


def test_roofline(line):
    r = line["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in r, k
    assert r["bound"] in ("hbm", "tensor") and r["unit"] == "GB/s"
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"], rel=1e-6)
    # algorithmic bytes: x read, y read and written, 16 B per ComplexF64 element, 64 kets
    assert r["algorithmic_bytes_per_launch"] == 3 * 16384 * 16 * 64
    assert r["achieved"] == pytest.approx(r["algorithmic_bytes_per_launch"] / (line["ms_per_step"] * 1e-3) / 1e9,
                                          rel=1e-6)
    f = line["fp64_compute"]
    assert f["frac"] == pytest.approx(f["achieved"] / f["peak"], rel=1e-6)


def test_end_to_end_and_cpu_baseline(line):
    e = line["e2e"]
    for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"):
        assert k in e, k
    nbytes = 64 * 16384 * 16
    assert e["h2d_bytes_per_step"] == 2 * nbytes and e["d2h_bytes_per_step"] == nbytes
    assert e["unit"] == line["unit"] and 0 < e["value"] < line["value"]
    c = line["cpu_baseline"]
    for k in ("value", "unit", "cores", "kind", "sample"):
        assert k in c, k
    assert c["kind"] in ("port", "reference") and c["cores"] >= 1 and c["value"] > 0


def test_clock_record_has_no_disqualifying_reason(line):
    c = line["clocks"]
    assert c["sm_mhz"] > 0 and c["sm_max_mhz"] > 0
    for bad in ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"):
        assert bad not in c["reasons"]


def test_other_forms_batched_and_served(line):
    for k in ("fp32_mode", "ff_mode"):
        assert line[k]["value"] > 0 and line[k]["ms_per_step"] > 0
    assert line["fp32_mode"]["rel_l2_err_vs_oracle"]["batch"] < 1e-5
    assert line["ff_mode"]["rel_l2_err_vs_oracle"]["batch"] < 1e-12
    assert line["rel_l2_err_vs_oracle"]["batch"] < 1e-12
    b = line["batched"]
    for k in ("complex128", "complex64", "complex128 double-float"):
        assert b[k]["applies_per_s"] > 0
    s = line["served"]
    for k in ("complex128", "complex64", "complex128 double-float"):
        assert s[k]["p50_ms"] <= s[k]["p99_ms"] and s[k]["sustained_applies_per_s"] > 0
    assert s["fp32_rel_err_vs_fp64_max"] < 1e-5
