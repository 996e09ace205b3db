"""The measured per-unit figures `bench.py` reads for its rooflines.

`bench.py` turns ncu counts of each dominant kernel (frozen in
`profiles/*.json`) into `roofline.traffic` and `roofline.issue`, and the
algorithmic counts (`oracle/flops.py`) into `roofline.fp32`.  These tests
check on the CPU that every file the bench reads exists with the fields it
uses, in ranges a capture of these kernels can give, and that the roofline
helpers turn them into fractions below 1 for the measured times."""

import importlib.util
import json
import pathlib

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


def _bench():
    spec = importlib.util.spec_from_file_location("bench_module", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _load(name):
    return json.loads((ROOT / "profiles" / name).read_text())


def test_trace_profile_fields():
    p = _load("trace_precision_1e8.json")
    for k in ("dram_bytes_per_ray", "algorithmic_flops_per_ray", "warp_instructions_per_32_rays",
              "flops_per_ray", "fma_pipe_active_pct", "algorithmic_div_per_ray",
              "algorithmic_special_per_ray"):
        assert isinstance(p[k], (int, float)) and p[k] > 0, k
    # streamed once: measured DRAM bytes at most the algorithmic 57 B/ray
    assert 40 < p["dram_bytes_per_ray"] <= p["algorithmic_bytes_per_ray"]
    # executed FP32 work exceeds the reference's (float-float compensation)
    assert p["flops_per_ray"] > p["algorithmic_flops_per_ray"]
    assert 32 * 20 < p["warp_instructions_per_32_rays"] < 32 * 100


@pytest.mark.parametrize("name, unit_bytes", [("multilayer_periodic_1e7.json", 28),
                                              ("trace_batch_spectrograph_256cfg.json", 13)])
def test_workload_profile_fields(name, unit_bytes):
    p = _load(name)
    assert p["algorithmic_bytes_per_unit"] == unit_bytes
    assert 0 < p["dram_bytes_per_unit"] <= unit_bytes
    assert p["warp_instructions_per_unit"] > 0
    assert p["executed_flops_per_unit"] == pytest.approx(
        p["fp32_fadd_per_unit"] + 2 * p["fp32_ffma_per_unit"] + p["fp32_fmul_per_unit"], rel=1e-3)


def test_roofline_helpers_give_fractions_below_one():
    b = _bench()
    pk = {"hbm_gbs": 6764.7, "sm_max_mhz": 2070.0}
    # the measured times of the configured workloads
    ml_fp32 = b.fp32_roofline("multilayer-periodic", 10_000_000, 4.52, pk)
    ml = b.issue_roofline("multilayer_periodic_1e7", 10_000_000, 4.52, pk, ml_fp32)
    bt_fp32 = b.fp32_roofline("batched-spectrograph", 606_601_488, 33.6, pk)
    bt = b.issue_roofline("trace_batch_spectrograph_256cfg", 606_601_488, 33.6, pk, bt_fp32)
    for r in (ml_fp32, ml, bt_fp32, bt):
        assert r is not None and 0 < r["frac"] < 1
    # the binding resource is instruction issue, far above the FP32 fraction
    assert ml["frac"] > 5 * ml_fp32["frac"] and bt["frac"] > 5 * bt_fp32["frac"]
    assert b._ncu_traffic("multilayer_periodic_1e7", 10) == pytest.approx(
        10 * _load("multilayer_periodic_1e7.json")["dram_bytes_per_unit"])
    assert b.issue_roofline("no_such_profile", 1, 1.0, pk, None) is None


def test_reference_arm_line(tmp_path):
    """`bench.py --impl reference` (the oracle on the host cores) prints one
    JSON line with the fields the comparison reads, on a small sample."""
    import subprocess
    import sys

    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps",
                        "1", "--warmup", "0", "--ref-rays", "4000"],
                       capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["unit"] == "rays*surfaces/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["cpu_baseline"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"],
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
