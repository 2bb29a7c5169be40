"""CPU-only checks of the benchmark's bookkeeping: the algorithmic flop count of one
gradient evaluation (14 per sector amplitude and target gate, 44 per fitted gate, 8 for
the overlap), the HBM view of the dominant kernel, and the command line."""
import os
import sys

import pytest

from conftest import ROOT

if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_alg_flops_headline():
    # L=16, 3336 target gates, 40 fitted gates, all 2^16 columns: 2^31 (14*3336 + 44*40 + 8)
    f = bench.alg_flops(16, 3336, 40, 1 << 16)
    assert f == float(1 << 31) * (14 * 3336 + 44 * 40 + 8)
    assert abs(f - 1.041e14) / 1.041e14 < 1e-3


def test_hbm_view():
    assert bench.hbm_view(None, 1.0) is None
    v = bench.hbm_view(328e9, 0.5)
    assert abs(v["achieved_gbs"] - 656.0) < 1e-9
    assert v["peak_source"] in ("measured", "fallback")
    assert abs(v["frac"] - v["achieved_gbs"] / v["peak_gbs"]) < 1e-15
    if not os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")):
        assert v["peak_gbs"] == 6800.0 and v["peak_source"] == "fallback"


@pytest.mark.parametrize("argv,want", [([], ("grad16", "per-gate", 3, 3)),
                                       (["--config", "hess14", "--hessian", "ti", "--steps", "5", "--warmup", "4"],
                                        ("hess14", "ti", 5, 4))])
def test_command_line(monkeypatch, argv, want):
    monkeypatch.setattr(sys, "argv", ["bench.py"] + argv)
    a = bench.parse()
    assert (a.config, a.hessian, a.steps, a.warmup) == want
    assert a.gpus == 1 and a.impl == "gb300"


def test_reference_arm_line(monkeypatch, capsys):
    """--impl reference on a small instance: ms_per_step is the wall time each step really
    took (steps x ms_per_step fits inside the run), the column sample is stated, and the
    config dict is the one the GPU arm prints"""
    import json
    import time
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--L", "8", "--layers", "4",
                                      "--trotter-steps", "2", "--steps", "2", "--warmup", "3"])
    t0 = time.perf_counter()
    bench.main()
    wall = time.perf_counter() - t0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["steps"] == 2 and line["warmup"] == 3
    assert line["steps"] * line["ms_per_step"] / 1e3 <= wall
    assert 0 < line["columns_per_step"] <= 256
    g, w, v, perms = bench.workload(8, 4, 2)
    assert line["config"] == bench.headline_config(8, 4, len(g), 2)
    assert abs(line["value"] - line["columns_per_step"] / 256 / (line["ms_per_step"] / 1e3)) < 1e-9 * line["value"]
