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
