"""The oracle against the reference library itself, compiled from the reference's own
sources by oracle/build_oracle.py, on seeded random instances (both driven through C).
Skipped where the reference checkout is absent."""
import ctypes as C

import numpy as np
import pytest

from conftest import brickwall_perms, crandn, random_gates, udist

import mgcu


def _hash(helpers):
    return mgcu.ufunc_address(helpers.mgt_hash_ufunc)


@pytest.mark.parametrize("L,i,j", [(6, 0, 1), (6, 4, 1), (7, 2, 5), (7, 6, 0), (8, 3, 4)])
def test_gate_kernels(oracle, reflib, L, i, j):
    rng = np.random.default_rng(L * 100 + i * 10 + j)
    g = random_gates(1, rng)[0]
    psi = crandn(1 << L, rng); d = crandn(1 << L, rng)
    assert udist(oracle.apply_gate(g, i, j, L, psi), reflib.apply_matchgate(g, i, j, psi)) < 1e-14
    dp1, dg1 = oracle.apply_gate_backward(g, i, j, L, psi, d)
    dp2, dg2 = reflib.apply_matchgate_backward(g, i, j, psi, d)
    assert udist(dp1, dp2) < 1e-14 and udist(dg1, dg2) < 1e-12
    arr = crandn(((1 << L), 8), rng)
    assert udist(oracle.apply_gate_array(g, i, j, L, arr), reflib.apply_matchgate_to_array(g, i, j, arr)) < 1e-14
    assert udist(oracle.apply_gate_backward_array(g, i, j, L, arr, d), reflib.apply_matchgate_backward_array(g, i, j, arr, d)) < 1e-12
    assert udist(oracle.apply_placeholder(i, j, L, psi), reflib.apply_placeholder(i, j, psi)) == 0


@pytest.mark.parametrize("L,nl,ti", [(6, 3, False), (6, 4, True), (8, 3, False)])
def test_brickwall_sweeps(oracle, reflib, L, nl, ti):
    rng = np.random.default_rng(7 + L + nl)
    v = random_gates(nl, rng)
    perms = brickwall_perms(L, nl, rng)
    psi = crandn(1 << L, rng); d = crandn(1 << L, rng)
    assert udist(oracle.brickwall_apply(v, perms, L, psi), reflib.brickwall_apply(v, perms, psi)) < 1e-13
    o1, c1 = oracle.brickwall_forward(v, perms, L, psi)
    o2, c2 = reflib.brickwall_forward(v, perms, psi)
    assert udist(o1, o2) < 1e-13 and udist(c1, c2) < 1e-13
    dp1, dv1 = oracle.brickwall_backward(v, perms, L, c1, d)
    dp2, dv2 = reflib.brickwall_backward(v, perms, c1, d)
    assert udist(dp1, dp2) < 1e-13 and udist(dv1, dv2) < 1e-12
    dp1, dv1, h1 = oracle.brickwall_backward_hessian(v, perms, L, c1, d, ti=ti)
    dp2, dv2, h2 = reflib.brickwall_backward(v, perms, c1, d, hessian=True, ti=ti)
    assert udist(dp1, dp2) < 1e-13 and udist(dv1, dv2) < 1e-12 and udist(h1, h2) < 1e-12


def test_circuit_target_and_gradient(oracle, reflib, helpers):
    rng = np.random.default_rng(3)
    L, ng = 7, 9
    gates = random_gates(ng, rng)
    wires = np.array([rng.choice(L, 2, replace=False) for _ in range(ng)], np.int32)
    t = oracle.Target("hash", L)
    f1, dg1 = oracle.circuit_target_and_gradient(t, gates, wires, L)
    rc, f2, dg2 = reflib.circuit_target_and_gradient(_hash(helpers), None, gates, wires, L)
    assert rc == 0
    assert abs(f1 - f2) < 1e-12 and udist(dg1, dg2) < 1e-11
    rc, f3 = reflib.circuit_target(_hash(helpers), None, gates, wires, L)
    assert abs(oracle.circuit_target(t, gates, wires, L) - f3) < 1e-12


@pytest.mark.parametrize("L,nl", [(6, 3), (8, 4)])
def test_brickwall_target_gradient_hessian(oracle, reflib, helpers, L, nl):
    rng = np.random.default_rng(L * nl)
    v = random_gates(nl, rng)
    perms = brickwall_perms(L, nl, rng)
    t = oracle.Target("hash", L)
    rc, f_r, dv_r, h_r = reflib.brickwall_target_gradient_hessian(_hash(helpers), None, v, perms, L)
    assert rc == 0
    f, dv, h = oracle.brickwall_target_gradient_hessian(t, v, perms, L)
    assert abs(f - f_r) < 1e-11 and udist(dv, dv_r) < 1e-11 and udist(h, h_r) < 1e-11
    rc, f_r2, dv_r2 = reflib.brickwall_target_and_gradient(_hash(helpers), None, v, perms, L)
    f2, dv2 = oracle.brickwall_target_and_gradient(t, v, perms, L)
    assert abs(f2 - f_r2) < 1e-11 and udist(dv2, dv_r2) < 1e-11
    rc, f_r3 = reflib.brickwall_target(_hash(helpers), None, v, perms, L)
    assert abs(oracle.brickwall_target(t, v, perms, L) - f_r3) < 1e-11


def test_ti_hessian_vs_reference(oracle, reflib, helpers):
    rng = np.random.default_rng(11)
    L, nl = 6, 4
    v = random_gates(nl, rng)
    perms = brickwall_perms(L, nl)
    U = crandn((1 << L, 1 << L), rng)
    Uc = np.ascontiguousarray(U)
    rc, f_r, dv_r, h_r = reflib.brickwall_target_gradient_hessian(mgcu.ufunc_address(helpers.mgt_dense_ufunc), Uc.ctypes.data, v, perms, L, ti=True)
    assert rc == 0
    f, dv, h = oracle.brickwall_target_gradient_hessian(oracle.Target("dense", L, U=U), v, perms, L, ti=True)
    assert abs(f - f_r) < 1e-11 and udist(dv, dv_r) < 1e-11 and udist(h, h_r) < 1e-11


def test_gradvec_hessmat(oracle, reflib, helpers):
    rng = np.random.default_rng(5)
    L, nl = 6, 3
    v = random_gates(nl, rng, unitary=True)
    perms = brickwall_perms(L, nl, rng)
    rc, f_r, g_r, H_r = reflib.brickwall_gradvec_hessmat(_hash(helpers), None, v, perms, L)
    assert rc == 0
    f, g, H = oracle.brickwall_gradvec_hessmat(oracle.Target("hash", L), v, perms, L)
    assert abs(f - f_r) < 1e-11 and udist(g, g_r) < 1e-11 and udist(H, H_r) < 1e-11


def test_algebra_and_tcg(oracle, reflib):
    rng = np.random.default_rng(9)
    for _ in range(5):
        a = random_gates(1, rng, scale=1.0)[0]
        assert udist(oracle.mg_polar(a), reflib.polar(a)) < 1e-14
        u = random_gates(1, rng, unitary=True)[0]
        eta = 0.3 * rng.standard_normal(8)
        # the reference retraction runs on the host there; compare the oracle with it
        z = np.zeros((1, 8), complex)
        reflib.lib.retract_matchgate(C.c_void_p(u.ctypes.data), C.c_void_p(eta.ctypes.data), C.c_void_p(z.ctypes.data))
        assert udist(oracle.mg_retract(u, eta), z[0]) < 1e-14
        zt = random_gates(1, rng, scale=1.0)[0]
        assert udist(oracle.mg_project_tangent(u, zt), reflib.project_tangent(u, zt)) < 1e-15
    n = 24
    A = rng.standard_normal((n, n)); H = A + A.T
    g = rng.standard_normal(n)
    for radius in [0.05, 1.0, 100.0]:
        z1, b1 = oracle.truncated_cg(g, H, radius, 2 * n)
        z2, b2 = reflib.truncated_cg(g, H, radius, 2 * n)
        assert b1 == b2 and udist(z1, z2) < 1e-12


def test_trust_region_vs_reference(oracle, reflib):
    """the reference's own optimiser driver (src/mg_brickwall_opt.c:99-122) on a
    brickwall target vs the oracle's trust-region loop"""
    rng = np.random.default_rng(21)
    L, nl, ul = 6, 3, 4
    perms = brickwall_perms(L, nl)
    uperms = brickwall_perms(L, ul)
    ulist = random_gates(ul, rng, unitary=True)
    v0 = random_gates(nl, rng, unitary=True)
    niter = 4
    f_o, fc_o, v_o = oracle.rtr_brickwall(oracle.Target("brickwall", L, ulist=ulist, uperms=uperms), v0, perms, L, niter)
    # the reference's optimize_matchgate_brickwall_circuit_hmat with the reference's own
    # brickwall application as the target map
    U = np.stack([oracle.brickwall_apply(ulist, uperms, L, e) for e in np.eye(1 << L)], axis=1)
    from conftest import ROOT  # noqa: F401
    helpers_lib = C.CDLL(reflib.path)  # same library
    prm = mgcu.RtrParams()
    prm.tcg_params = mgcu.TcgParams(2 * 16 * nl, 1e-8, 1e-6)
    prm.rho_trust, prm.radius_init, prm.maxradius = 0.125, 0.01, 0.1
    f_iter = np.zeros(niter + 1); f_citer = np.zeros(niter + 1, complex); vo = np.zeros_like(v0)
    pp, rows = mgcu._perm_ptrs(perms, L)
    import os
    so = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "libmgtest.so")
    dense = C.CDLL(so).mgt_dense_ufunc
    Uc = np.ascontiguousarray(U)
    v0 = np.ascontiguousarray(v0)
    helpers_lib.optimize_matchgate_brickwall_circuit_hmat(C.c_void_p(mgcu.ufunc_address(dense)), C.c_void_p(Uc.ctypes.data),
                                                          C.c_void_p(v0.ctypes.data), nl, L, C.cast(pp, C.c_void_p), C.byref(prm), niter,
                                                          C.c_void_p(f_iter.ctypes.data), C.c_void_p(f_citer.ctypes.data),
                                                          C.c_void_p(vo.ctypes.data))
    assert np.max(np.abs(f_iter - f_o)) < 1e-9
    assert udist(vo, v_o) < 1e-9
