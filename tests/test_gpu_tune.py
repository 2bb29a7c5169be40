"""The target sweep's block size chosen by timing (MG_OPT_TARGET_TUNE): every candidate
applies the same operations to each amplitude in the same order, so plans that tuned and
plans that did not must give bit-identical f and gradients, for the weight-restricted sweep
(a Hubbard Trotter target) and the full sweep (Haar matchgate brickwall target), and the
chosen configuration must be one of the candidates."""
import os
import sys

import numpy as np
import pytest

import mgcu
import targets as T

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402

pytestmark = pytest.mark.gpu


def _run(lib, t, v, perms, L, tune):
    lib.set_option(mgcu.OPT_TARGET_TUNE, tune)
    try:
        plan = lib.plan_brickwall(lib.mg_target_apply, t, v, perms, L, mgcu.EVAL_GRADIENT)
    finally:
        lib.set_option(mgcu.OPT_TARGET_TUNE, 0)
    try:
        cfg = lib.plan_target_config(plan)
        assert lib.lib.mg_plan_run(mgcu.P(plan)) == 0, lib.last_error()
        f, dv, _, _, _ = lib.plan_results(plan, len(v), grad=True)
    finally:
        lib.lib.mg_plan_free(mgcu.P(plan))
    return cfg, f, dv


@pytest.mark.parametrize("kind,L,prec", [("hubbard", 12, mgcu.PREC_MIXED), ("hubbard", 14, mgcu.PREC_FP64),
                                         ("haar", 12, mgcu.PREC_MIXED), ("haar", 14, mgcu.PREC_FP32)])
def test_tuned_sweep_is_bit_identical(mglib, kind, L, prec):
    lib = mglib
    rng = np.random.default_rng(L + prec)
    if kind == "hubbard":
        g, w, v, perms = bench.workload(L, 3, 4, seed=L)
        t = lib.target_circuit(g, w, L)
    else:
        ul, up = T.haar_matchgates(6, rng), T.brickwall_perms(L, 6)
        v, perms = T.haar_matchgates(3, rng), T.brickwall_perms(L, 3)
        t = lib.target_brickwall(ul, up, L)
    lib.set_precision(prec)
    try:
        c1, f1, dv1 = _run(lib, t, v, perms, L, 1)   # the static choice
        c2, f2, dv2 = _run(lib, t, v, perms, L, 2)   # timed
        c3, f3, dv3 = _run(lib, t, v, perms, L, 2)   # the cached choice
    finally:
        lib.set_precision(mgcu.PREC_FP64)
        lib.target_free(t)
    assert c1["kind"] == (2 if kind == "hubbard" else 1)
    assert c2 == c3 and c2["kind"] == c1["kind"] and c2["tile_bits"] == c1["tile_bits"]
    if c2["kind"] == 2:
        assert (c2["threads"], c2["per_thread"]) in [(128, 2), (256, 1)]
    else:
        assert c2["threads"] in (128, 256, 512)
    assert f1 == f2 == f3
    assert np.array_equal(dv1, dv2) and np.array_equal(dv1, dv3)
