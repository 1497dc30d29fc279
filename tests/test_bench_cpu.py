"""The benchmark's host-side bookkeeping, without a GPU: the algorithmic-bytes
model, the per-launch figures it reads from the committed ncu summaries for its
roofline objects, and the peak it divides by."""
import json

import pytest

import bench

GATHERS = ("density_high", "density_low", "force_low", "force_high")


@pytest.mark.parametrize("fname", ["dram_traffic.txt", "warp_instructions.txt"])
def test_profile_tables_cover_every_gather_of_the_headline_workload(fname):
    """bench.py's `traffic` and `issue_roofline` read these tables for the
    developed 1M dam break, in both arithmetics; every gather must have a row."""
    for arith in ("exact", "fast"):
        for stage in GATHERS:
            v = bench._profile_value(fname, "dam_break_1m_developed", arith, stage)
            assert v is not None and v > 0, (fname, arith, stage)
    assert bench._profile_value(fname, "no_such_workload", "exact", "force_high") is None


def test_issue_roofline_arithmetic():
    inst = bench._profile_value("warp_instructions.txt", "dam_break_1m_developed", "exact", "force_high")
    r = bench.issue_roofline("dam_break_1m_developed", "exact", "force_high", 0.1, 2070.0)
    assert r["warp_inst_per_launch"] == inst
    assert r["achieved"] == pytest.approx(inst / 1e-4)
    sms = r["peak"] / (4.0 * 2070.0e6)
    assert sms == pytest.approx(round(sms))  # 4 warp instructions per SM per cycle
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert bench.issue_roofline("dam_break_1m_developed", "exact", "force_high", None, 2070.0) is None


def test_stage_bytes_model():
    """Per-particle and per-cell bytes of each stage, as the design notes state
    them: own state read and written once per dependent pass, the neighbour lists
    written by the densities (25 B) and read by the forces."""
    n_low, n_high, c_low, c_high = 1000, 2000, 300, 1200
    nb = bench.NBR_BYTES
    assert bench.stage_bytes("density_low", n_low, n_high, c_low, c_high, False, 0) == n_low * (21 + nb) + 4 * c_low
    assert bench.stage_bytes("density_high", n_low, n_high, c_low, c_high, False, 0) == n_high * (21 + nb) + 4 * c_high
    assert bench.stage_bytes("force_low", n_low, n_high, c_low, c_high, False, 0) == n_low * (59 + nb) + 4 * c_low
    assert bench.stage_bytes("force_high", n_low, n_high, c_low, c_high, True, 0) == n_high * (78 + nb + 12) + 4 * c_low
    assert bench.stage_bytes("grid_low", n_low, n_high, c_low, c_high, False, 0) == n_low * 85 + 12 * c_low
    assert bench.stage_bytes("relax", n_low, n_high, c_low, c_high, True, 40, relax_iters=4) == 40 * 4 * 56
    assert bench.stage_bytes("no_such_stage", n_low, n_high, c_low, c_high, False, 0) == 0


def test_hbm_peak_reads_the_measured_file_or_says_fallback(tmp_path, monkeypatch):
    p = tmp_path / "peaks.json"
    p.write_text(json.dumps({"hbm_gbs": 6793.8, "bf16_tflops": 1900.0}))
    monkeypatch.setattr(bench, "MEASURED_PEAKS", str(p))
    assert bench.hbm_peak() == (6793.8, "measured")
    monkeypatch.setattr(bench, "MEASURED_PEAKS", str(tmp_path / "absent.json"))
    assert bench.hbm_peak() == (bench.FALLBACK_HBM_GBS, "fallback")
