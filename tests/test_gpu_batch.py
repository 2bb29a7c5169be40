"""Batches (mg_batch_*): many brickwall fits of different qubit counts and depths in one
persistent launch per phase, replayed from a captured CUDA graph, against one-instance
evaluations of the same library and against the oracle."""
import numpy as np
import pytest

import mgcu
from conftest import random_gates

pytestmark = pytest.mark.gpu


def _perms(L, nl):
    even = np.arange(L)
    odd = np.roll(np.arange(L), -1)
    return np.array([even if i % 2 == 0 else odd for i in range(nl)], np.int32)


def _instances(lib, shapes, seed):
    """(L, fitted depth) -> random brickwall target of twice the depth, random fit"""
    rng = np.random.default_rng(seed)
    out = []
    for L, nl in shapes:
        ul = random_gates(2 * nl, rng, unitary=True)
        t = lib.target_brickwall(ul, _perms(L, 2 * nl), L)
        out.append({"L": L, "nl": nl, "t": t, "v": random_gates(nl, rng, unitary=True), "perms": _perms(L, nl),
                    "ul": ul})
    return out


SHAPES = [(10, 3), (12, 5), (14, 4), (10, 9), (12, 6), (8, 7)]


@pytest.mark.parametrize("prec", [mgcu.PREC_FP64, mgcu.PREC_MIXED])
def test_batch_matches_single_instances(mglib, prec):
    lib = mglib
    inst = _instances(lib, SHAPES, 7)
    lib.set_precision(prec)
    try:
        b = lib.batch_create([x["t"] for x in inst], [x["v"] for x in inst], [x["perms"] for x in inst], [x["L"] for x in inst])
        assert lib.batch_run(b) == 0, lib.last_error()
        res = [lib.batch_results(b, i) for i in range(len(inst))]
        # deterministic replay
        assert lib.batch_run(b) == 0
        res2 = [lib.batch_results(b, i) for i in range(len(inst))]
        for (f, dv, g), (f2, dv2, g2) in zip(res, res2):
            assert f == f2 and np.array_equal(dv, dv2) and np.array_equal(g, g2)
        for i, x in enumerate(inst):
            kt, npass, items = lib.batch_info(b, i)
            assert 5 <= kt <= 13 and npass >= 1 and items >= 1
            rc, f1, dv1 = lib.brickwall_target_and_gradient(lib.mg_target_apply, x["t"], x["v"], x["perms"], x["L"])
            assert rc == 0
            rc, fp, gp = lib.brickwall_projected_gradient(lib.mg_target_apply, x["t"], x["v"], x["perms"], x["L"])
            f, dv, g = res[i]
            s = max(1.0, abs(f1))
            assert abs(f - f1) < 1e-12 * s, (i, f, f1)
            assert np.max(np.abs(dv - dv1)) < 1e-12 * max(1.0, np.max(np.abs(dv1)))
            assert np.max(np.abs(g - gp)) < 1e-12 * max(1.0, np.max(np.abs(gp)))
        # new gates for one instance, then a replay of the same graph
        rng = np.random.default_rng(11)
        x = inst[1]
        x["v"] = random_gates(x["nl"], rng, unitary=True)
        assert lib.batch_set_gates(b, 1, x["v"]) == 0
        assert lib.batch_run(b) == 0
        f, dv, g = lib.batch_results(b, 1)
        rc, f1, dv1 = lib.brickwall_target_and_gradient(lib.mg_target_apply, x["t"], x["v"], x["perms"], x["L"])
        assert abs(f - f1) < 1e-12 * max(1.0, abs(f1)) and np.max(np.abs(dv - dv1)) < 1e-12 * max(1.0, np.max(np.abs(dv1)))
        lib.batch_free(b)
    finally:
        lib.set_precision(mgcu.PREC_FP64)
        for x in inst:
            lib.target_free(x["t"])


def test_batch_vs_oracle(mglib, oracle):
    lib = mglib
    inst = _instances(lib, [(8, 3), (10, 4)], 3)
    lib.set_precision(mgcu.PREC_FP64)
    try:
        b = lib.batch_create([x["t"] for x in inst], [x["v"] for x in inst], [x["perms"] for x in inst],
                             [x["L"] for x in inst], tune=False)
        assert lib.batch_run(b) == 0
        for i, x in enumerate(inst):
            f, dv, _ = lib.batch_results(b, i)
            tgt = oracle.Target("brickwall", x["L"], ulist=x["ul"], uperms=_perms(x["L"], 2 * x["nl"]))
            f_o, dv_o = oracle.brickwall_target_and_gradient(tgt, x["v"], x["perms"], x["L"])
            assert abs(f - f_o) < 1e-12 * max(1.0, abs(f_o)) and np.max(np.abs(dv - dv_o)) < 1e-12 * max(1.0, np.max(np.abs(dv_o)))
        lib.batch_free(b)
    finally:
        for x in inst:
            lib.target_free(x["t"])


def test_batch_rejects_host_targets(mglib, helpers):
    lib = mglib
    rng = np.random.default_rng(1)
    with pytest.raises(RuntimeError):
        lib.batch_create([mgcu.ufunc_address(helpers.mgt_hash_ufunc)], [random_gates(2, rng)], [_perms(8, 2)], [8])
