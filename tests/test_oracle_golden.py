"""The oracle (C restatement of the reference) against the reference's own golden
vectors, regenerated by tests/golden/gen_golden.py.  Tolerances are the reference
tests' (test/test_gate.c, test/test_matchgate*.c)."""
import numpy as np
import pytest

from conftest import udist

MAP16 = [5, 6, 9, 10, 0, 3, 12, 15]   # matchgate entry -> general 4x4 entry (test/test_gate.c:384)


def test_apply_gate(oracle, golden):
    g = golden("test_apply_matchgate_cplx")
    v = g.gate("v/center", "v/corner")
    psi = g.c("psi")
    for (i, j), k in [((2, 5), "chi1"), ((4, 1), "chi2"), ((3, 4), "chi3")]:
        assert udist(oracle.apply_gate(v, i, j, 9, psi), g.c(k)) < 1e-12


def test_apply_gate_array(oracle, golden):
    g = golden("test_apply_matchgate_to_array_cplx")
    v = g.gate("v/center", "v/corner")
    psi = g.c("psi")
    for (i, j), k in [((2, 5), "chi1"), ((4, 1), "chi2"), ((3, 4), "chi3")]:
        assert udist(oracle.apply_gate_array(v, i, j, 6, psi), g.c(k)) < 1e-12


def test_backward_array_consistent(oracle, golden):
    """test/test_gate.c:209-284: array gradients equal single-vector gradients"""
    g = golden("test_apply_matchgate_backward_array_cplx")
    v = g.gate("v/center", "v/corner")
    arr = g.c("psi_array")
    d = g.c("dpsi_out")
    for i, j in zip([2, 3, 4, 7, 5], [5, 4, 1, 6, 8]):
        dgs = oracle.apply_gate_backward_array(v, i, j, 9, arr, d)
        for s in range(8):
            _, dg = oracle.apply_gate_backward(v, i, j, 9, g.c(f"psi{s}"), d)
            assert udist(dgs[s], dg) < 1e-12


def test_backward_finite_difference(oracle, golden):
    """test/test_gate.c:130-206: Wirtinger derivatives against finite differences"""
    g = golden("test_apply_matchgate_backward_cplx")
    v = g.gate("v/center", "v/corner")
    psi, dout = g.c("psi"), g.c("dpsi_out")
    h = 1e-5
    for i, j in [(2, 5), (3, 4), (4, 1)]:
        dpsi, dg = oracle.apply_gate_backward(v, i, j, 9, psi, dout)
        # f(V) = <dout, G(V) psi> (bilinear): df/dV_e = dg[e]
        for e in range(8):
            dv = np.zeros(8, complex); dv[e] = h
            fp = np.sum(dout * oracle.apply_gate(v + dv, i, j, 9, psi))
            fm = np.sum(dout * oracle.apply_gate(v - dv, i, j, 9, psi))
            assert abs((fp - fm) / (2 * h) - dg[e]) < 1e-8
        # df/dpsi_a = dpsi[a]
        for a in [0, 17, 300, 511]:
            dp = np.zeros(512, complex); dp[a] = h
            fp = np.sum(dout * oracle.apply_gate(v, i, j, 9, psi + dp))
            fm = np.sum(dout * oracle.apply_gate(v, i, j, 9, psi - dp))
            assert abs((fp - fm) / (2 * h) - dpsi[a]) < 1e-8


def test_placeholder(oracle, golden):
    g = golden("test_apply_matchgate_placeholder_cplx")
    psi = g.c("psi")
    for (i, j), k in [((2, 5), "psi_out1"), ((5, 1), "psi_out2")]:
        ref16 = g.c(k).reshape(128, 16)
        out8 = oracle.apply_placeholder(i, j, 7, psi)
        assert udist(out8, ref16[:, MAP16]) < 1e-12


def test_brickwall_apply(oracle, golden):
    g = golden("test_apply_matchgate_brickwall_unitary_cplx")
    v = np.array([g.gate(f"v/center{i}", f"v/corner{i}") for i in range(4)])
    perms = np.array([g[f"perm{i}"] for i in range(4)])
    psi = g.c("psi")
    for k, nl in enumerate([3, 4]):
        assert udist(oracle.brickwall_apply(v[:nl], perms[:nl], 8, psi), g.c(f"chi{k}")) < 1e-12


def test_brickwall_forward_backward(oracle, golden):
    g = golden("test_matchgate_brickwall_unitary_backward_cplx")
    v = np.array([g.gate(f"v/center{i}", f"v/corner{i}") for i in range(4)])
    perms = np.array([g[f"perm{i}"] for i in range(4)])
    psi, dout = g.c("psi"), g.c("dpsi_out")
    for k, nl in enumerate([3, 4]):
        out, cache = oracle.brickwall_forward(v[:nl], perms[:nl], 6, psi)
        assert udist(out, g.c(f"psi_out{k}")) < 1e-12
        dpsi, dv = oracle.brickwall_backward(v[:nl], perms[:nl], 6, cache, dout)
        # f(V) = <dout, W(V) psi>; dv[l] is its derivative w.r.t. the shared gate of layer l
        h = 1e-5
        for l in range(nl):
            for e in [0, 3, 5, 6]:
                vp = v[:nl].copy(); vp[l, e] += h
                vm = v[:nl].copy(); vm[l, e] -= h
                num = (np.sum(dout * oracle.brickwall_apply(vp, perms[:nl], 6, psi)) -
                       np.sum(dout * oracle.brickwall_apply(vm, perms[:nl], 6, psi))) / (2 * h)
                assert abs(num - dv[l, e]) < 1e-8


def test_circuit_target(oracle, golden):
    g = golden("test_matchgate_circuit_unitary_target_cplx")
    gates = np.array([g.gate(f"G/center{i}", f"G/corner{i}") for i in range(5)])
    f = oracle.circuit_target(oracle.Target("hash", 7), gates, g["wires"], 7)
    assert abs(f - g.c("f")) < 1e-12


def test_brickwall_target(oracle, golden):
    g = golden("test_matchgate_brickwall_unitary_target_cplx")
    v = np.array([g.gate(f"V/center{i}", f"V/corner{i}") for i in range(5)])
    perms = np.array([g[f"perm{i}"] for i in range(5)])
    t = oracle.Target("hash", 8)
    for k, nl in enumerate([4, 5]):
        assert abs(oracle.brickwall_target(t, v[:nl], perms[:nl], 8) - g.c(f"f{k}")) < 1e-12


def test_brickwall_target_gradient_hessian(oracle, golden):
    """test/test_matchgate_target.c:219-388 (f, gradients 1e-12, Hessian symmetry 1e-12)"""
    g = golden("test_matchgate_brickwall_unitary_target_gradient_hessian_cplx")
    v = np.array([g.gate(f"V/center{i}", f"V/corner{i}") for i in range(5)])
    perms = np.array([g[f"perm{i}"] for i in range(5)])
    t = oracle.Target("hash", 6)
    for k, nl in enumerate([4, 5]):
        f, dv, hess = oracle.brickwall_target_gradient_hessian(t, v[:nl], perms[:nl], 6)
        assert abs(f - g.c(f"f{k}")) < 1e-12
        dv_ref = np.array([g.gate(f"dVlist{k}/center{i}", f"dVlist{k}/corner{i}") for i in range(nl)])
        assert udist(dv, dv_ref) < 1e-12
        assert udist(hess, hess.T) < 1e-12
        # the same gradient through the target-and-gradient path
        f2, dv2 = oracle.brickwall_target_and_gradient(t, v[:nl], perms[:nl], 6)
        assert abs(f2 - f) < 1e-12 and udist(dv2, dv) < 1e-12


def test_gradvec_hessmat(oracle, golden):
    """test/test_matchgate_target.c:390-500: f 1e-12, grad 1e-14, H 1e-13, H symmetric"""
    g = golden("test_matchgate_brickwall_unitary_target_gradient_vector_hessian_matrix_cplx")
    v = np.array([g.gate(f"V/center{i}", f"V/corner{i}") for i in range(5)])
    perms = np.array([g[f"perm{i}"] for i in range(5)])
    f, grad, H = oracle.brickwall_gradvec_hessmat(oracle.Target("hash", 6), v, perms, 6)
    assert abs(f - g.c("f")) < 1e-12
    assert udist(grad, g["grad"]) < 1e-13
    assert udist(H, H.T) < 1e-14
    assert udist(H.reshape(-1), g["H"]) < 1e-12


def test_ti_matches_plain(oracle, golden):
    """test/test_matchgate_target.c:506-590: translation-invariant Hessian equals the plain
    one for a translation-invariant target and brickwall"""
    g = golden("test_matchgate_ti_brickwall_unitary_target_gradient_hessian_cplx")
    v = np.array([g.gate(f"V/center{i}", f"V/corner{i}") for i in range(7)])
    perms = np.array([g[f"perm{i}"] for i in range(7)])
    t = oracle.Target("dense", 8, U=g.c("expiH"))
    f1, dv1, h1 = oracle.brickwall_target_gradient_hessian(t, v, perms, 8, ti=False)
    f2, dv2, h2 = oracle.brickwall_target_gradient_hessian(t, v, perms, 8, ti=True)
    assert abs(f1 - f2) < 1e-12
    assert udist(dv1, dv2) < 1e-12
    assert udist(h1, h2) < 1e-13


def test_algebra(oracle, golden):
    g = golden("test_multiply_matchgate_cplx")
    c = oracle.mg_multiply(g.gate("a/center", "a/corner"), g.gate("b/center", "b/corner"))
    assert udist(c, g.gate("c/center", "c/corner")) < 1e-14
    g = golden("test_project_tangent_matchgate_cplx")
    p = oracle.mg_project_tangent(g.gate("u/center", "u/corner"), g.gate("z/center", "z/corner"))
    assert udist(p, g.gate("p/center", "p/corner")) < 1e-14
    g = golden("test_polar_matchgate_factor_cplx")
    u = oracle.mg_polar(g.gate("a/center", "a/corner"))
    assert udist(u, g.gate("u/center", "u/corner")) < 1e-13
    # test/test_matchgate.c:150-210: real_to_tangent(tangent_to_real(v, t), v) is the
    # tangent projection of t at the unitary v
    g = golden("test_real_to_tangent_matchgate_cplx")
    v, t = g.gate("v/center", "v/corner"), g.gate("t/center", "t/corner")
    r = oracle.mg_tangent_to_real(v, t)
    assert udist(oracle.mg_real_to_tangent(r, v), oracle.mg_project_tangent(v, t)) < 1e-14
