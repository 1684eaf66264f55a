"""The arithmetic behind bench.py's numbers, on the CPU: stored-mode
dimensions, algorithmic bytes and flops (the roofline numerators), the
summary of the clock samples, the per-band errors and the ensemble's
members."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_stored_mode_dimensions_follow_the_two_thirds_rule():
    # k_max = int((N - 0.1) / 3): Nx_min = k + 1, Ny_min = Nz_min = 2 k + 1
    assert bench.dims(256) == (86, 171, 171)
    assert bench.dims(128) == (43, 85, 85)
    assert bench.dims(96) == (32, 63, 63)
    assert bench.dims(32) == (11, 21, 21)


def test_x_pass_bytes_are_the_pencils_read_and_written():
    # Lu + Lr = 13 fields of Nx_min x N x N complex values, read or written once
    assert bench.x_pass_bytes(256, 8) == 16 * 13 * 86 * 256 * 256 == 1_172_307_968
    assert bench.x_pass_bytes(256, 4) == 586_153_984
    assert bench.x_pass_flops(256) == pytest.approx(5 * 256 * 8 * 13 * 256 * 128)


def test_step_bytes_match_the_documented_totals():
    # 14.3 GB per FP64 step and 7.2 GB per FP32 step at 256^3
    assert bench.algorithmic_bytes_per_step(256, 8) / 1e9 == pytest.approx(14.3, abs=0.05)
    assert bench.algorithmic_bytes_per_step(256, 4) * 2 == bench.algorithmic_bytes_per_step(256, 8)


def test_clock_summary_reports_the_median_clock_and_throttle_reasons():
    c = bench.Clocks()
    c.samples = [["2070", "2070", "900.5", "Not Active", "Not Active", "Not Active", "Not Active"],
                 ["1980", "2070", "1350.0", "Not Active", "Not Active", "Not Active", "Active"],
                 ["2070", "2070", "1200.0", "Not Active", "Not Active", "Not Active", "Not Active"],
                 ["[N/A]", "2070"],  # unreadable lines are skipped
                 ]
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"] and s["samples"] == 3
    assert bench.Clocks().summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_band_errors(monkeypatch):
    monkeypatch.setattr(bench, "N", 32)
    mx, my, mz = bench.dims()
    rng = np.random.default_rng(0)
    shape = (mz + 2, my, mx, 2)  # Nze rows: the padding rows are ignored
    ref = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    same = bench.band_errors(ref.copy(), ref)
    assert all(v == 0.0 for row in same.values() for v in row.values())
    scaled = bench.band_errors(ref * (1 + 1e-6), ref)
    for row in scaled.values():
        assert len(row) == 3
        for v in row.values():
            assert v == pytest.approx(1e-6, rel=1e-6)


def test_ensemble_members():
    members = bench.ensemble_members()
    assert len(members) == 96
    sizes = [cfg["nx"] for cfg, _, _ in members]
    assert [sizes.count(n) for n in (32, 64, 96, 128)] == [32, 32, 24, 8]
    for cfg, seed, learned in members:
        assert cfg["nx"] == cfg["ny"] == cfg["nz"]
        assert 0.25 <= cfg["buoy_fac_z"] <= 16.0  # N^2, N uniform in [0.5, 4]
        assert 0.5 / 150 <= cfg["vis"] <= 0.5 / 50  # Re_lambda uniform in [50, 150]
        assert learned == (cfg["nx"] >= 96)
    assert bench.ensemble_members() == members  # seeded
