"""The gradient sweep without per-gate caches (k_columns_adj, MG_OPT_FIT_CACHE=2, for callers
short of device memory): the forward sweep keeps each pass's output state and the backward
sweep recovers every fitted gate's input with the gate's block inverses.  It must agree with
the cached sweep (MG_OPT_FIT_CACHE=1, the reference's method, src/matchgate_brickwall.c:
52-127) and with the oracle, and a fitted gate that has no inverse must fall back to the
cache."""
import numpy as np
import pytest

import mgcu
import targets as T
from conftest import random_gates

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("L,nl,prec,tol", [(12, 5, mgcu.PREC_MIXED, 1e-11), (14, 4, mgcu.PREC_MIXED, 1e-11),
                                           (14, 6, mgcu.PREC_FP32, 1e-4), (10, 3, mgcu.PREC_MIXED, 1e-11),
                                           (8, 4, mgcu.PREC_MIXED, 1e-11), (6, 3, mgcu.PREC_FP32, 1e-4)])
def test_checkpointed_sweep_matches_cached(mglib, oracle, L, nl, prec, tol):
    lib = mglib
    rng = np.random.default_rng(300 + L + nl)
    ul, up = T.haar_matchgates(2 * nl, rng), T.brickwall_perms(L, 2 * nl)
    v = random_gates(nl, rng, unitary=True)
    perms = T.brickwall_perms(L, nl)
    t = lib.target_brickwall(ul, up, L)
    out = []
    lib.set_precision(prec)
    try:
        for cache in (2, 1):   # checkpointed, then cached
            lib.set_option(mgcu.OPT_FIT_CACHE, cache)
            out.append(lib.brickwall_columns(lib.mg_target_apply, t, v, perms, L, 0, min(200, 1 << L)))
    finally:
        lib.set_option(mgcu.OPT_FIT_CACHE, 0)
        lib.set_precision(mgcu.PREC_FP64)
        lib.target_free(t)
    (rc0, f0, dv0), (rc1, f1, dv1) = out
    assert rc0 == 0 and rc1 == 0
    f_o, dv_o = oracle.brickwall_target_and_gradient(oracle.Target("brickwall", L, ulist=ul, uperms=up), v, perms, L,
                                                     col_range=(0, min(200, 1 << L)))
    for f, dv in ((f0, dv0), (f1, dv1)):
        assert abs(f - f_o) <= tol * abs(f_o)
        assert np.linalg.norm(dv - dv_o) <= tol * np.linalg.norm(dv_o)


def test_singular_fitted_gate_uses_the_cache(mglib, oracle):
    """a fitted block with no inverse (a projector): the sweep falls back to cached inputs"""
    lib = mglib
    L, nl = 10, 3
    rng = np.random.default_rng(31)
    ul, up = T.haar_matchgates(6, rng), T.brickwall_perms(L, 6)
    v = random_gates(nl, rng, unitary=True)
    v[1, 4:] = [1, 0, 0, 0]   # corner block diag(1, 0)
    perms = T.brickwall_perms(L, nl)
    t = lib.target_brickwall(ul, up, L)
    lib.set_precision(mgcu.PREC_MIXED)
    lib.set_option(mgcu.OPT_FIT_CACHE, 2)
    try:
        rc, f, dv = lib.brickwall_columns(lib.mg_target_apply, t, v, perms, L, 0, 1 << L)
    finally:
        lib.set_option(mgcu.OPT_FIT_CACHE, 0)
        lib.set_precision(mgcu.PREC_FP64)
        lib.target_free(t)
    assert rc == 0, lib.last_error()
    f_o, dv_o = oracle.brickwall_target_and_gradient(oracle.Target("brickwall", L, ulist=ul, uperms=up), v, perms, L)
    assert abs(f - f_o) <= 1e-11 * abs(f_o)
    assert np.linalg.norm(dv - dv_o) <= 1e-11 * np.linalg.norm(dv_o)
