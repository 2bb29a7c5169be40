"""Per-gate Riemannian gradient and Hessian (one parameter block per gate, the reference's
per-layer projection of src/matchgate_target.c:877-973 applied gate by gate) and the
trust-region fit on them.  No reference fixture covers the per-gate forms, so they are
pinned three ways: (1) a brickwall written as a circuit, its per-gate blocks summed over each
layer, equals the per-layer forms of the oracle; (2) finite differences of f along the
retraction curve R(x, t eta) give g.eta and eta.H.eta (the polar retraction is of second
order); (3) the per-gate trust region decreases f, and float-float follows complex128."""
import numpy as np
import pytest

import mgcu
import targets as T

pytestmark = pytest.mark.gpu


def _brickwall_as_circuit(v, perms, L):
    half = L // 2
    gates = np.array([v[l] for l in range(len(v)) for _ in range(half)])
    wires = np.array([[perms[l][2 * p], perms[l][2 * p + 1]] for l in range(len(v)) for p in range(half)], np.int32)
    return gates, wires


def test_per_gate_forms_sum_to_per_layer_oracle(mglib, oracle):
    lib = mglib
    lib.set_precision(mgcu.PREC_FP64)
    L, nl, nu = 8, 4, 6
    rng = np.random.default_rng(81)
    v = T.haar_matchgates(nl, rng)
    perms = T.brickwall_perms(L, nl)
    ul, up = T.haar_matchgates(nu, rng), T.brickwall_perms(L, nu)
    gates, wires = _brickwall_as_circuit(v, perms, L)
    t = lib.target_brickwall(ul, up, L)
    try:
        rc, f, gv, H = lib.circuit_gradvec_hessmat(lib.mg_target_apply, t, gates, wires, L)
        rc2, f2, gv2 = lib.circuit_projected_gradient(lib.mg_target_apply, t, gates, wires, L)
    finally:
        lib.target_free(t)
    assert rc == 0 and rc2 == 0, lib.last_error()
    f_o, g_o, H_o = oracle.brickwall_gradvec_hessmat(oracle.Target("brickwall", L, ulist=ul, uperms=up), v, perms, L)
    half = L // 2
    S = np.zeros((8 * nl, 8 * len(gates)))   # sums the gates of each layer
    for g in range(len(gates)):
        for x in range(8):
            S[8 * (g // half) + x, 8 * g + x] = 1
    assert abs(f - f_o) < 1e-12 * abs(f_o)
    assert np.max(np.abs(S @ gv - g_o)) < 1e-11 * np.max(np.abs(g_o))
    assert np.max(np.abs(S @ H @ S.T - H_o)) < 1e-11 * np.max(np.abs(H_o))
    assert np.max(np.abs(gv - gv2)) < 1e-13 * np.max(np.abs(gv))
    assert np.max(np.abs(H - H.T)) < 1e-11 * np.max(np.abs(H))


def test_per_gate_forms_match_finite_differences(mglib):
    lib = mglib
    lib.set_precision(mgcu.PREC_FP64)
    L, nu = 8, 8
    rng = np.random.default_rng(82)
    # C1's open chain: 4 layers, 4 + 3 + 4 + 3 = 14 gates
    wires = np.array([[i, i + 1] for layer in range(4) for i in range(layer % 2, L - 1, 2)], np.int32)
    gates = T.haar_matchgates(len(wires), rng)
    ul, up = T.haar_matchgates(nu, rng), T.brickwall_perms(L, nu)
    t = lib.target_brickwall(ul, up, L)
    try:
        rc, f0, gv, H = lib.circuit_gradvec_hessmat(lib.mg_target_apply, t, gates, wires, L)
        assert rc == 0, lib.last_error()
        eta = rng.standard_normal(8 * len(gates))
        eta /= np.linalg.norm(eta)

        def f_at(s):
            x = np.array([lib.retract(gates[g], s * eta[8 * g:8 * g + 8]) for g in range(len(gates))])
            rc, f = lib.circuit_target(lib.mg_target_apply, t, x, wires, L)
            assert rc == 0
            return f.real
        h1, h2 = 1e-5, 1e-3
        d1 = (f_at(h1) - f_at(-h1)) / (2 * h1)
        d2 = (f_at(h2) - 2 * f0.real + f_at(-h2)) / h2 ** 2
    finally:
        lib.target_free(t)
    assert abs(d1 - gv @ eta) < 1e-6 * max(1.0, abs(gv @ eta))
    assert abs(d2 - eta @ H @ eta) < 1e-4 * max(1.0, abs(eta @ H @ eta))


def test_per_gate_trust_region(mglib):
    """C1's per-gate fit (14 gates, 112 real parameters) against a depth-8 random brickwall:
    f decreases over the accepted steps, and the float-float run follows complex128"""
    lib = mglib
    L = 8
    rng1, rng2 = np.random.default_rng(1), np.random.default_rng(2)
    wires = np.array([[i, i + 1] for layer in range(4) for i in range(layer % 2, L - 1, 2)], np.int32)
    gates0 = T.haar_matchgates(len(wires), rng1)
    ul, up = T.haar_matchgates(8, rng2), T.brickwall_perms(L, 8)
    t = lib.target_brickwall(ul, up, L)
    try:
        f64, p64, x64 = lib.optimize_circuit_native(t, gates0, wires, L, 8)
        fmx, pmx, xmx = lib.optimize_circuit_native(t, gates0, wires, L, 8, refine_gnorm=1e-300)
    finally:
        lib.target_free(t)
    assert np.all(p64 == mgcu.PREC_FP64) and np.all(pmx == mgcu.PREC_MIXED)
    assert np.all(np.diff(f64) <= 1e-9 * np.abs(f64[:-1]))   # the iterate only moves on accepted steps
    assert f64[-1] < f64[0]
    assert np.max(np.abs(fmx - f64) / np.abs(f64)) < 1e-8
    # the final gates stay unitary blocks
    for g in x64:
        for b in (g[:4].reshape(2, 2), g[4:].reshape(2, 2)):
            assert np.allclose(b.conj().T @ b, np.eye(2), atol=1e-12)
