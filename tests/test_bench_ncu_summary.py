"""bench.py's machine-written ncu summary (--ncu-json) and the lookup that
feeds roofline.traffic: raw-page CSVs (header row, units row, one row per
captured launch) summarised per kernel with the units of the second row
converted to nanoseconds and bytes, several files merged, launches
averaged; the profiled step's scope names mapped to the kernels ncu sees."""
import csv
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _raw(path, kernel, rows):
    head = ["ID", "Kernel Name", "gpu__time_duration.sum", "dram__bytes_read.sum", "dram__bytes_write.sum",
            "launch__registers_per_thread"]
    units = ["", "", "us", "Mbyte", "Kbyte", "register/thread"]
    with open(path, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(head)
        w.writerow(units)
        for n, (t, r, wr) in enumerate(rows):
            w.writerow([str(n), f"void game::(anonymous namespace)::{kernel}<float, 0>(HGrid<float>, int)",
                        f"{t}", f"{r}", f"{wr}", "72"])


def test_summary_scales_units_and_merges_files(tmp_path):
    a, b = tmp_path / "a.csv", tmp_path / "b.csv"
    _raw(a, "k_scalar_tend2", [(190.0, 180.0, 40.0), (200.0, 240.0, 50.0)])
    _raw(b, "k_tracers_solve_df", [(128.0, 145.0, 37.5)])
    out = tmp_path / "s.json"
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--ncu-json", str(a), str(b), "--out",
                        str(out), "--command", "cmd", "--captured", "what"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    d = json.loads(out.read_text())
    assert d["command"] == "cmd" and d["captured"] == "what"
    k = d["kernels"]["k_scalar_tend2"]
    assert k["launches"] == 2
    assert k["duration_ns"] == pytest.approx(195e3)
    assert k["dram_read_bytes"] == pytest.approx(210e6)
    assert k["dram_write_bytes"] == pytest.approx(45e3)
    assert k["dram_bytes_per_launch"] == pytest.approx(210e6 + 45e3)
    assert k["registers_per_thread"] == 72
    assert d["kernels"]["k_tracers_solve_df"]["duration_ns"] == pytest.approx(128e3)


def test_traffic_lookup_maps_scope_names_to_kernels(tmp_path, monkeypatch):
    prof = tmp_path / "p.json"
    prof.write_text(json.dumps({"commit": "abc", "captured": "x", "kernels": {
        "k_scalar_tend2": {"dram_bytes_per_launch": 2.5e8},
        "k_tracers_solve_df": {"dram_bytes_per_launch": 1.8e8}}}))
    monkeypatch.setattr(bench, "PROFILE_JSON", str(prof))
    v, src = bench.read_profile("k_scalar_tend", "dram_bytes_per_launch")
    assert v == 2.5e8 and src["commit"] == "abc"
    v, _ = bench.read_profile("k_tracers_solve", "dram_bytes_per_launch")
    assert v == 1.8e8
    assert bench.read_profile("k_waves_rows", "dram_bytes_per_launch") == (None, None)


def test_short_kernel_names():
    assert bench.short_kernel_name("void game::(anonymous namespace)::k_waves_thomas_df<26>(int, WavesWork)") \
        == "k_waves_thomas_df"
    assert bench.short_kernel_name("k_theta(int, int)") == "k_theta"
