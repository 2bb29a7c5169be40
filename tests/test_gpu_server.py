"""Request server (mg_server_*): continuous batching of f, gradient, Hessian and
trust-region-step requests; each result is the same alone and in a mix (complex128: 1e-12
relative, float-float: 1e-9, the summation order differs), with a step's Hessian and
trust-region requests served on a second stream beside its batch, and the HBM budget admits
requests."""
import threading
import time

import numpy as np
import pytest

import mgcu
from conftest import random_gates

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _perms(L, nl):
    even = np.arange(L)
    odd = np.roll(np.arange(L), -1)
    return np.array([even if i % 2 == 0 else odd for i in range(nl)], np.int32)


def _requests(lib, seed):
    rng = np.random.default_rng(seed)
    kinds = [mgcu.REQ_TARGET, mgcu.REQ_GRADIENT, mgcu.REQ_HESSIAN, mgcu.REQ_TRSTEP, mgcu.REQ_GRADIENT,
             mgcu.REQ_TARGET, mgcu.REQ_GRADIENT, mgcu.REQ_TRSTEP]
    Ls = [10, 8, 8, 8, 12, 12, 10, 10]
    out = []
    for k, L in zip(kinds, Ls):
        nl = int(rng.integers(3, 6))
        t = lib.target_brickwall(random_gates(2 * nl, rng, unitary=True), _perms(L, 2 * nl), L)
        out.append({"kind": k, "L": L, "nl": nl, "t": t, "v": random_gates(nl, rng, unitary=True), "perms": _perms(L, nl),
                    "radius": 0.05})
    return out


def _submit(lib, sv, x):
    return lib.server_submit(sv, x["kind"], x["t"], x["v"], x["perms"], x["L"], x["radius"])


def _same(a, b, kind, tol=TOL):
    s = max(1.0, abs(b["f"]))
    assert a["status"] == 0 and b["status"] == 0
    assert abs(a["f"] - b["f"]) < tol * s
    if kind != mgcu.REQ_TARGET:
        assert np.max(np.abs(a["grad_vec"] - b["grad_vec"])) < tol * max(1.0, np.max(np.abs(b["grad_vec"])))
    if kind in (mgcu.REQ_HESSIAN, mgcu.REQ_TRSTEP):
        assert np.max(np.abs(a["H"] - b["H"])) < tol * max(1.0, np.max(np.abs(b["H"])))
    if kind == mgcu.REQ_TRSTEP:
        assert a["accepted"] == b["accepted"] and a["radius"] == b["radius"]
        assert np.max(np.abs(a["vlist"] - b["vlist"])) < 1e2 * tol


@pytest.mark.parametrize("prec,tol", [(mgcu.PREC_FP64, TOL), (mgcu.PREC_MIXED, 1e-9)])
def test_server_mix_equals_alone(mglib, prec, tol):
    lib = mglib
    lib.set_precision(prec)
    reqs = _requests(lib, 5)
    try:
        sv = lib.server_create(120 << 30)
        alone = []
        for x in reqs:                       # one request per step
            rid = _submit(lib, sv, x)
            alone.append(lib.server_result(sv, rid, x["nl"]))
        steps0, _, _ = lib.server_stats(sv)
        assert steps0 == len(reqs)
        # the same requests submitted together from two threads: served in few steps
        ids = [None] * len(reqs)

        def sub(idx):
            for i in idx:
                ids[i] = _submit(lib, sv, reqs[i])
        th = [threading.Thread(target=sub, args=(range(k, len(reqs), 2),)) for k in (0, 1)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        mixed = [lib.server_result(sv, ids[i], x["nl"]) for i, x in enumerate(reqs)]
        steps1, batched, peak = lib.server_stats(sv)
        assert steps1 - steps0 < len(reqs) and batched > len([x for x in reqs if x["kind"] <= 1])
        for a, b, x in zip(mixed, alone, reqs):
            _same(a, b, x["kind"], tol)
        # the alone results against the one-instance API
        for r, x in zip(alone, reqs):
            if x["kind"] == mgcu.REQ_GRADIENT:
                rc, f, g = lib.brickwall_projected_gradient(lib.mg_target_apply, x["t"], x["v"], x["perms"], x["L"])
                assert rc == 0 and abs(r["f"] - f) < tol * max(1, abs(f)) and np.max(np.abs(r["grad_vec"] - g)) < tol * max(1, np.max(np.abs(g)))
            if x["kind"] == mgcu.REQ_HESSIAN:
                rc, f, g, H = lib.brickwall_gradvec_hessmat(lib.mg_target_apply, x["t"], x["v"], x["perms"], x["L"])
                assert rc == 0 and np.max(np.abs(r["H"] - H)) < tol * max(1, np.max(np.abs(H)))
            t = r["times"]
            assert t[0] <= t[1] <= t[2]
        lib.server_free(sv)
    finally:
        lib.set_precision(mgcu.PREC_FP64)
        for x in reqs:
            lib.target_free(x["t"])


def test_server_budget_admission(mglib):
    lib = mglib
    lib.set_precision(mgcu.PREC_FP64)
    allr = _requests(lib, 9)
    reqs = [x for x in allr if x["kind"] == mgcu.REQ_GRADIENT]
    try:
        # device workspace estimate of a gradient request (the server's formula): staged
        # target columns plus per-block slots and gate cache; a budget just above the
        # largest one serves the three requests in at least two steps
        def est(x):
            S, N, G = 1 << (x["L"] - 1), 1 << x["L"], x["nl"] * x["L"] // 2
            return min(N * S * 16, 16 << 30) + 304 * (2 + G) * S * 16
        budget = max(est(x) for x in reqs) + (1 << 20)
        assert sum(est(x) for x in reqs) > budget
        sv = lib.server_create(budget)
        ids = [_submit(lib, sv, x) for x in reqs]
        res = [lib.server_result(sv, i, x["nl"]) for i, x in zip(ids, reqs)]
        assert all(r["status"] == 0 for r in res)
        steps, batched, peak = lib.server_stats(sv)
        assert steps >= 2 and 0 < peak <= budget
        lib.server_free(sv)
        # a request that can never fit fails with -6
        sv = lib.server_create(1 << 20)
        rid = _submit(lib, sv, reqs[0])
        assert lib.server_result(sv, rid, reqs[0]["nl"])["status"] == -6
        lib.server_free(sv)
    finally:
        for x in allr:
            lib.target_free(x["t"])
