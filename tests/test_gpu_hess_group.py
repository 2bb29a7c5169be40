"""The plain per-layer Hessian by grouped forward-mode items (MG_OPT_HESS_GROUP 0: one sweep
per column, layer and entry that adds the placeholder term of each of the layer's gates as it
passes them) against the reference's per-gate placements (MG_OPT_HESS_GROUP 1,
src/matchgate_brickwall.c:177-231) and against the oracle: the same pairs of gates contribute
to the same Hessian blocks, so the two agree to rounding.  The translation-invariant Hessian
and the per-gate Hessian keep one item per placement gate and are unaffected."""
import numpy as np
import pytest

import mgcu
import targets as T

pytestmark = pytest.mark.gpu


def _rel(x, y):
    return float(np.linalg.norm(np.asarray(x) - np.asarray(y)) / max(np.linalg.norm(np.asarray(y)), 1e-300))


@pytest.mark.parametrize("L,nl,prec,tol", [(8, 3, mgcu.PREC_FP64, 1e-12), (10, 5, mgcu.PREC_FP64, 1e-12),
                                           (12, 4, mgcu.PREC_MIXED, 1e-9), (12, 6, mgcu.PREC_FP64, 1e-12),
                                           (14, 3, mgcu.PREC_MIXED, 1e-9), (10, 4, mgcu.PREC_FP32, 2e-4)])
def test_grouped_hessian_matches_per_gate_placements(mglib, L, nl, prec, tol):
    lib = mglib
    rng = np.random.default_rng(L * 10 + nl)
    ul, up = T.haar_matchgates(2 * nl, rng), T.brickwall_perms(L, 2 * nl)
    v = T.haar_matchgates(nl, rng)
    perms = T.brickwall_perms(L, nl)
    t = lib.target_brickwall(ul, up, L)
    lib.set_precision(prec)
    out = []
    try:
        for grp in (0, 1):
            lib.set_option(mgcu.OPT_HESS_GROUP, grp)
            out.append((lib.brickwall_target_gradient_hessian(lib.mg_target_apply, t, v, perms, L),
                        lib.brickwall_gradvec_hessmat(lib.mg_target_apply, t, v, perms, L)))
    finally:
        lib.set_option(mgcu.OPT_HESS_GROUP, 0)
        lib.set_precision(mgcu.PREC_FP64)
        lib.target_free(t)
    (h0, p0), (h1, p1) = out
    assert h0[0] == 0 and h1[0] == 0 and p0[0] == 0 and p1[0] == 0, lib.last_error()
    assert h0[1] == h1[1] and np.array_equal(h0[2], h1[2])   # f and the gradient do not involve the items
    assert _rel(h0[3], h1[3]) <= tol
    assert _rel(p0[3], p1[3]) <= tol and np.array_equal(p0[2], p1[2])
    assert np.max(np.abs(h0[3] - h0[3].T)) <= tol * np.max(np.abs(h0[3]))


@pytest.mark.parametrize("L,nl", [(8, 4), (10, 3)])
def test_grouped_hessian_vs_oracle(mglib, oracle, L, nl):
    lib = mglib
    lib.set_precision(mgcu.PREC_FP64)
    rng = np.random.default_rng(7 + L)
    ul, up = T.haar_matchgates(2 * nl, rng), T.brickwall_perms(L, 2 * nl)
    v = T.haar_matchgates(nl, rng)
    perms = T.brickwall_perms(L, nl)
    t = lib.target_brickwall(ul, up, L)
    try:
        rc, f, dv, h = lib.brickwall_target_gradient_hessian(lib.mg_target_apply, t, v, perms, L)
        rc2, f2, g2, H2 = lib.brickwall_gradvec_hessmat(lib.mg_target_apply, t, v, perms, L)
    finally:
        lib.target_free(t)
    assert rc == 0 and rc2 == 0, lib.last_error()
    t_o = oracle.Target("brickwall", L, ulist=ul, uperms=up)
    f_o, dv_o, h_o = oracle.brickwall_target_gradient_hessian(t_o, v, perms, L)
    f2_o, g_o, H_o = oracle.brickwall_gradvec_hessmat(t_o, v, perms, L)
    assert abs(f - f_o) <= 1e-12 * abs(f_o)
    assert _rel(dv, dv_o) <= 1e-12 and _rel(h, h_o) <= 1e-12
    assert _rel(g2, g_o) <= 1e-12 and _rel(H2, H_o) <= 1e-12
