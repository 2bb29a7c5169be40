"""GPU parity: the library (through its C API) against the reference's golden vectors
and against the oracle, in complex128.  Tolerances are the reference tests' own
(states, f and gradients 1e-12; real Hessian 1e-13; symmetry 1e-12/1e-14)."""
import numpy as np
import pytest

import mgcu
from conftest import brickwall_perms, crandn, random_gates, udist

pytestmark = pytest.mark.gpu

MAP16 = [5, 6, 9, 10, 0, 3, 12, 15]


@pytest.fixture(scope="module")
def lib(mglib):
    mglib.set_precision(mgcu.PREC_FP64)
    for o in (1, 2, 3, 4):
        mglib.set_option(o, 0)
    return mglib


def _hash(helpers):
    return mgcu.ufunc_address(helpers.mgt_hash_ufunc)


# ------------------------------------------------------------------ single gates (gate.h)
def test_apply_matchgate_golden(lib, golden):
    g = golden("test_apply_matchgate_cplx")
    v = g.gate("v/center", "v/corner")
    for (i, j), k in [((2, 5), "chi1"), ((4, 1), "chi2"), ((3, 4), "chi3")]:
        assert udist(lib.apply_matchgate(v, i, j, g.c("psi")), g.c(k)) < 1e-12


def test_apply_to_array_golden(lib, golden):
    g = golden("test_apply_matchgate_to_array_cplx")
    v = g.gate("v/center", "v/corner")
    for (i, j), k in [((2, 5), "chi1"), ((4, 1), "chi2"), ((3, 4), "chi3")]:
        assert udist(lib.apply_matchgate_to_array(v, i, j, g.c("psi")), g.c(k)) < 1e-12


def test_placeholders_golden(lib, golden):
    g = golden("test_apply_matchgate_placeholder_cplx")
    for (i, j), k in [((2, 5), "psi_out1"), ((5, 1), "psi_out2")]:
        ref16 = g.c(k).reshape(128, 16)
        assert udist(lib.apply_placeholder(i, j, g.c("psi"), nout=16), ref16) < 1e-12
        assert udist(lib.apply_placeholder(i, j, g.c("psi"), nout=8), ref16[:, MAP16]) < 1e-12


def test_backward_and_array_vs_oracle(lib, oracle, golden):
    g = golden("test_apply_matchgate_backward_array_cplx")
    v = g.gate("v/center", "v/corner")
    arr, d = g.c("psi_array"), g.c("dpsi_out")
    for i, j in zip([2, 3, 4, 7, 5], [5, 4, 1, 6, 8]):
        dp, dg = lib.apply_matchgate_backward(v, i, j, g.c("psi0"), d)
        dp_o, dg_o = oracle.apply_gate_backward(v, i, j, 9, g.c("psi0"), d)
        assert udist(dp, dp_o) < 1e-12 and udist(dg, dg_o) < 1e-12
        assert udist(lib.apply_matchgate_backward_array(v, i, j, arr, d), oracle.apply_gate_backward_array(v, i, j, 9, arr, d)) < 1e-12


# ------------------------------------------------------------------ sweeps on one vector
def test_brickwall_apply_golden(lib, golden):
    g = golden("test_apply_matchgate_brickwall_unitary_cplx")
    v = np.array([g.gate(f"v/center{i}", f"v/corner{i}") for i in range(4)])
    perms = np.array([g[f"perm{i}"] for i in range(4)])
    for k, nl in enumerate([3, 4]):
        assert udist(lib.brickwall_apply(v[:nl], perms[:nl], g.c("psi")), g.c(f"chi{k}")) < 1e-12


@pytest.mark.parametrize("ti", [False, True])
def test_brickwall_backward_hessian_golden(lib, oracle, golden, ti):
    g = golden("test_matchgate_brickwall_unitary_backward_hessian_cplx")
    v = np.array([g.gate(f"v/center{i}", f"v/corner{i}") for i in range(4)])
    perms = np.array([g[f"perm{i}"] for i in range(4)])
    psi, d = g.c("psi"), g.c("dpsi_out")
    for k, nl in enumerate([1, 2, 3, 4]):
        out, cache = lib.brickwall_forward(v[:nl], perms[:nl], psi)
        assert udist(out, g.c(f"psi_out{k}")) < 1e-12
        dp, dv = lib.brickwall_backward(v[:nl], perms[:nl], cache, d)
        dp_o, dv_o = oracle.brickwall_backward(v[:nl], perms[:nl], 6, cache, d)
        assert udist(dp, dp_o) < 1e-12 and udist(dv, dv_o) < 1e-12
        dp, dv, h = lib.brickwall_backward(v[:nl], perms[:nl], cache, d, hessian=True, ti=ti)
        dp_o, dv_o, h_o = oracle.brickwall_backward_hessian(v[:nl], perms[:nl], 6, cache, d, ti=ti)
        assert udist(dp, dp_o) < 1e-12 and udist(dv, dv_o) < 1e-12 and udist(h, h_o) < 1e-12


def test_circuit_sweeps_vs_oracle(lib, oracle):
    rng = np.random.default_rng(4)
    L, ng = 7, 11
    gates = random_gates(ng, rng)
    wires = np.array([rng.choice(L, 2, replace=False) for _ in range(ng)], np.int32)
    psi, d = crandn(1 << L, rng), crandn(1 << L, rng)
    assert udist(lib.circuit_apply(gates, wires, psi), oracle.circuit_apply(gates, wires, L, psi)) < 1e-12
    out, cache = lib.circuit_forward(gates, wires, psi)
    dp, dg = lib.circuit_backward(gates, wires, cache, d)
    # oracle: per-gate gradients of f = <d, C psi>
    h = 1e-6
    for gi in [0, 5, 10]:
        for e in [1, 6]:
            gp = gates.copy(); gp[gi, e] += h
            gm = gates.copy(); gm[gi, e] -= h
            num = (np.sum(d * oracle.circuit_apply(gp, wires, L, psi)) - np.sum(d * oracle.circuit_apply(gm, wires, L, psi))) / (2 * h)
            assert abs(num - dg[gi, e]) < 1e-7


# ------------------------------------------------------------------ traces (matchgate_target.h)
def test_circuit_target_golden(lib, golden, helpers):
    g = golden("test_matchgate_circuit_unitary_target_cplx")
    gates = np.array([g.gate(f"G/center{i}", f"G/corner{i}") for i in range(5)])
    rc, f = lib.circuit_target(_hash(helpers), None, gates, g["wires"], 7)
    assert rc == 0 and abs(f - g.c("f")) < 1e-12


def test_brickwall_target_golden(lib, golden, helpers):
    g = golden("test_matchgate_brickwall_unitary_target_cplx")
    v = np.array([g.gate(f"V/center{i}", f"V/corner{i}") for i in range(5)])
    perms = np.array([g[f"perm{i}"] for i in range(5)])
    for k, nl in enumerate([4, 5]):
        rc, f = lib.brickwall_target(_hash(helpers), None, v[:nl], perms[:nl], 8)
        assert rc == 0 and abs(f - g.c(f"f{k}")) < 1e-12


@pytest.mark.parametrize("parallel", [False, True])
def test_target_gradient_hessian_golden(lib, oracle, golden, helpers, parallel):
    g = golden("test_matchgate_brickwall_unitary_target_gradient_hessian_cplx")
    v = np.array([g.gate(f"V/center{i}", f"V/corner{i}") for i in range(5)])
    perms = np.array([g[f"perm{i}"] for i in range(5)])
    t = oracle.Target("hash", 6)
    for k, nl in enumerate([4, 5]):
        rc, f, dv, h = lib.brickwall_target_gradient_hessian(_hash(helpers), None, v[:nl], perms[:nl], 6, parallel=parallel)
        assert rc == 0
        assert abs(f - g.c(f"f{k}")) < 1e-12
        dv_ref = np.array([g.gate(f"dVlist{k}/center{i}", f"dVlist{k}/corner{i}") for i in range(nl)])
        assert udist(dv, dv_ref) < 1e-12
        assert udist(h, h.T) < 1e-12
        _, _, h_o = oracle.brickwall_target_gradient_hessian(t, v[:nl], perms[:nl], 6)
        assert udist(h, h_o) < 1e-12
        rc, f2, dv2 = lib.brickwall_target_and_gradient(_hash(helpers), None, v[:nl], perms[:nl], 6)
        assert rc == 0 and abs(f2 - f) < 1e-12 and udist(dv2, dv) < 1e-12


def test_gradvec_hessmat_golden(lib, golden, helpers):
    g = golden("test_matchgate_brickwall_unitary_target_gradient_vector_hessian_matrix_cplx")
    v = np.array([g.gate(f"V/center{i}", f"V/corner{i}") for i in range(5)])
    perms = np.array([g[f"perm{i}"] for i in range(5)])
    rc, f, grad, H = lib.brickwall_gradvec_hessmat(_hash(helpers), None, v, perms, 6)
    assert rc == 0
    assert abs(f - g.c("f")) < 1e-12
    assert udist(grad, g["grad"]) < 1e-13
    assert udist(H, H.T) < 1e-14
    assert udist(H.reshape(-1), g["H"]) < 1e-12
    rc, f2, grad2 = lib.brickwall_projected_gradient(_hash(helpers), None, v, perms, 6)
    assert rc == 0 and abs(f2 - f) < 1e-12 and udist(grad2, grad) < 1e-13


@pytest.mark.parametrize("name,nl,invariant", [("test_matchgate_ti_brickwall_unitary_target_gradient_hessian_cplx", 7, True),
                                               ("test_matchgate_ti_brickwall_unitary_target_gradient_hessian2_cplx", 5, False)])
def test_ti_hessian_golden(lib, oracle, golden, name, nl, invariant):
    """test/test_matchgate_target.c:506-673.  For the first fixture (translation-invariant
    target and periodic brickwall) the translation-invariant Hessian equals the plain one.
    The second fixture's wiring (test/permutations.py:121-133, spin blocks plus an
    interaction layer) is not covariant under the pair translation the shortcut assumes:
    there the reference's own two Hessians differ (by 0.0449), so both are checked against
    the oracle's restatement of the respective reference routine instead."""
    g = golden(name)
    U = g.c("expiH")
    L = 8
    if "V__center0" in g.d.files:
        v = np.array([g.gate(f"V/center{i}", f"V/corner{i}") for i in range(nl)])
    else:
        blocks = g.c("vlist")
        v = np.array([np.concatenate([blocks[2 * i].reshape(4), blocks[2 * i + 1].reshape(4)]) for i in range(nl)])
    perms = np.array([g[f"perm{i}"] for i in range(nl)])
    t = lib.target_dense(U, L)
    try:
        rc, f1, dv1, h1 = lib.brickwall_target_gradient_hessian(lib.mg_target_apply, t, v, perms, L)
        rc2, f2, dv2, h2 = lib.brickwall_target_gradient_hessian(lib.mg_target_apply, t, v, perms, L, ti=True)
    finally:
        lib.target_free(t)
    assert rc == 0 and rc2 == 0
    assert abs(f1 - f2) < 1e-12 and udist(dv1, dv2) < 1e-12
    if invariant:
        assert udist(h1, h2) < 1e-12
    ot = oracle.Target("dense", L, U=U)
    for ti, (f, dv, h) in [(False, (f1, dv1, h1)), (True, (f2, dv2, h2))]:
        f_o, dv_o, h_o = oracle.brickwall_target_gradient_hessian(ot, v, perms, L, ti=ti)
        assert abs(f - f_o) < 1e-12 and udist(dv, dv_o) < 1e-12 and udist(h, h_o) < 1e-12


# ------------------------------------------------------------------ GPU targets, larger sizes, tiling
@pytest.mark.parametrize("kind", ["brickwall", "circuit", "dense"])
def test_gpu_targets_vs_oracle(lib, oracle, kind):
    rng = np.random.default_rng({"brickwall": 1, "circuit": 2, "dense": 3}[kind])
    L, nl, ul = 8, 4, 8
    v = random_gates(nl, rng, unitary=True)
    perms = brickwall_perms(L, nl)
    if kind == "brickwall":
        ulist = random_gates(ul, rng, unitary=True); uperms = brickwall_perms(L, ul, rng)
        t = lib.target_brickwall(ulist, uperms, L)
        ot = oracle.Target("brickwall", L, ulist=ulist, uperms=uperms)
    elif kind == "circuit":
        ng = 30
        gates = random_gates(ng, rng, unitary=True)
        wires = np.array([rng.choice(L, 2, replace=False) for _ in range(ng)], np.int32)
        t = lib.target_circuit(gates, wires, L)
        ot = oracle.Target("circuit", L, gates=gates, wires=wires)
    else:
        U = crandn((1 << L, 1 << L), rng)
        t = lib.target_dense(U, L)
        ot = oracle.Target("dense", L, U=U)
    try:
        rc, f, dv, h = lib.brickwall_target_gradient_hessian(lib.mg_target_apply, t, v, perms, L)
        assert rc == 0
        f_o, dv_o, h_o = oracle.brickwall_target_gradient_hessian(ot, v, perms, L)
        assert abs(f - f_o) < 1e-12 * max(1, abs(f_o))
        assert udist(dv, dv_o) < 1e-11 and udist(h, h_o) < 1e-11
        # the target map itself on a host vector
        psi = crandn(1 << L, rng)
        out = np.zeros_like(psi)
        import ctypes as C
        a, b = mgcu.StateVector(psi.ctypes.data, L), mgcu.StateVector(out.ctypes.data, L)
        assert lib.lib.mg_target_apply(C.byref(a), C.c_void_p(t), C.byref(b)) == 0
        assert udist(out, ot.apply(psi)) < 1e-12
    finally:
        lib.target_free(t)


@pytest.mark.parametrize("L,nl,tile_bits", [(10, 5, 0), (10, 5, 5), (12, 3, 7), (12, 4, 0)])
def test_tiled_passes_vs_oracle(lib, oracle, L, nl, tile_bits):
    """several shared-memory tiles per column (tile_bits < L-1) against the oracle"""
    rng = np.random.default_rng(L + nl + tile_bits)
    v = random_gates(nl, rng, unitary=True)
    perms = brickwall_perms(L, nl, rng)
    ul = 6
    ulist = random_gates(ul, rng, unitary=True); uperms = brickwall_perms(L, ul, rng)
    t = lib.target_brickwall(ulist, uperms, L)
    lib.set_option(mgcu.OPT_TILE_BITS, tile_bits)
    try:
        rc, f, dv = lib.brickwall_target_and_gradient(lib.mg_target_apply, t, v, perms, L)
        assert rc == 0
        cols = (0, 1 << L) if L <= 10 else (0, 256)
        if L > 10:
            rc, f, dv = lib.brickwall_columns(lib.mg_target_apply, t, v, perms, L, *cols)
            assert rc == 0
        ot = oracle.Target("brickwall", L, ulist=ulist, uperms=uperms)
        f_o, dv_o = oracle.brickwall_target_and_gradient(ot, v, perms, L, col_range=cols)
        assert abs(f - f_o) < 1e-11 * max(1, abs(f_o))
        assert udist(dv, dv_o) < 1e-11 * max(1, np.max(np.abs(dv_o)))
    finally:
        lib.set_option(mgcu.OPT_TILE_BITS, 0)
        lib.target_free(t)


def test_tiled_hessian_vs_oracle(lib, oracle):
    rng = np.random.default_rng(77)
    L, nl = 10, 3
    v = random_gates(nl, rng, unitary=True)
    perms = brickwall_perms(L, nl, rng)
    U = crandn((1 << L, 1 << L), rng) / 32
    t = lib.target_dense(U, L)
    lib.set_option(mgcu.OPT_TILE_BITS, 6)
    try:
        rc, f, dv, h = lib.brickwall_target_gradient_hessian(lib.mg_target_apply, t, v, perms, L)
        rc2, f2, dv2, h2 = lib.brickwall_target_gradient_hessian(lib.mg_target_apply, t, v, perms, L, ti=True)
    finally:
        lib.set_option(mgcu.OPT_TILE_BITS, 0)
        lib.target_free(t)
    assert rc == 0 and rc2 == 0
    ot = oracle.Target("dense", L, U=U)
    f_o, dv_o, h_o = oracle.brickwall_target_gradient_hessian(ot, v, perms, L, nthreads=0)
    assert abs(f - f_o) < 1e-11 and udist(dv, dv_o) < 1e-11 and udist(h, h_o) < 1e-10
    _, _, h2_o = oracle.brickwall_target_gradient_hessian(ot, v, perms, L, ti=True)
    assert udist(h2, h2_o) < 1e-10


@pytest.mark.parametrize("prec", [mgcu.PREC_FP64, mgcu.PREC_MIXED])
def test_hessian_reduction_runs(lib, prec):
    """Hessian items reduce once per run of gates with the same block and weight, capped at
    64 quartets per thread: with 32 threads on a 2^11 tile (16 quartets per thread) a
    six-gate layer is cut after four gates, with 256 threads (2 per thread) it is one run.
    Both, and the translation-invariant weights, agree with each other; the uncapped path
    is checked against the oracle by the golden and tiled Hessian tests."""
    rng = np.random.default_rng(91)
    L, nl = 12, 3
    v = random_gates(nl, rng, unitary=True)
    perms = brickwall_perms(L, nl, rng)
    ulist = random_gates(4, rng, unitary=True)
    uperms = brickwall_perms(L, 4, rng)
    t = lib.target_brickwall(ulist, uperms, L)
    out = {}
    lib.set_precision(prec)
    try:
        for threads in (0, 32, 64):
            lib.set_option(mgcu.OPT_THREADS, threads)
            for ti in (False, True):
                rc, f, dv, h = lib.brickwall_target_gradient_hessian(lib.mg_target_apply, t, v, perms, L, ti=ti)
                assert rc == 0, lib.last_error()
                out[threads, ti] = (f, dv, h)
    finally:
        lib.set_option(mgcu.OPT_THREADS, 0)
        lib.set_precision(mgcu.PREC_FP64)
        lib.target_free(t)
    tol = 1e-12 if prec == mgcu.PREC_FP64 else 1e-9
    for ti in (False, True):
        f0, dv0, h0 = out[0, ti]
        for threads in (32, 64):
            f, dv, h = out[threads, ti]
            assert abs(f - f0) < tol * abs(f0) and udist(dv, dv0) < tol * np.max(np.abs(dv0))
            assert udist(h, h0) < tol * np.max(np.abs(h0))


def test_per_gate_circuit_gradient_and_hessian(lib, oracle, helpers):
    rng = np.random.default_rng(12)
    L, ng = 6, 8
    gates = random_gates(ng, rng)
    wires = np.array([rng.choice(L, 2, replace=False) for _ in range(ng)], np.int32)
    t = oracle.Target("hash", L)
    rc, f, dg = lib.circuit_target_and_gradient(_hash(helpers), None, gates, wires, L)
    f_o, dg_o = oracle.circuit_target_and_gradient(t, gates, wires, L)
    assert rc == 0 and abs(f - f_o) < 1e-12 and udist(dg, dg_o) < 1e-11
    rc, f, dg, h = lib.circuit_target_gradient_hessian(_hash(helpers), None, gates, wires, L)
    f_o, dg_o, h_o = oracle.circuit_target_gradient_hessian(t, gates, wires, L)
    assert rc == 0 and udist(dg, dg_o) < 1e-11 and udist(h, h_o) < 1e-11
    assert udist(h, h.T) < 1e-12


def test_column_ranges_sum_to_trace(lib, oracle):
    rng = np.random.default_rng(8)
    L, nl = 8, 3
    v = random_gates(nl, rng, unitary=True); perms = brickwall_perms(L, nl)
    ulist = random_gates(4, rng, unitary=True); uperms = brickwall_perms(L, 4, rng)
    t = lib.target_brickwall(ulist, uperms, L)
    try:
        rc, f, dv = lib.brickwall_target_and_gradient(lib.mg_target_apply, t, v, perms, L)
        parts = [lib.brickwall_columns(lib.mg_target_apply, t, v, perms, L, b0, b1) for b0, b1 in [(0, 37), (37, 200), (200, 256)]]
    finally:
        lib.target_free(t)
    assert all(p[0] == 0 for p in parts)
    assert abs(sum(p[1] for p in parts) - f) < 1e-12
    assert udist(sum(p[2] for p in parts), dv) < 1e-12


def test_deterministic(lib):
    rng = np.random.default_rng(99)
    L, nl = 10, 4
    v = random_gates(nl, rng, unitary=True); perms = brickwall_perms(L, nl)
    ulist = random_gates(8, rng, unitary=True); uperms = brickwall_perms(L, 8, rng)
    t = lib.target_brickwall(ulist, uperms, L)
    try:
        r1 = lib.brickwall_target_and_gradient(lib.mg_target_apply, t, v, perms, L)
        r2 = lib.brickwall_target_and_gradient(lib.mg_target_apply, t, v, perms, L)
    finally:
        lib.target_free(t)
    assert r1[1] == r2[1] and np.array_equal(r1[2], r2[2])


def test_error_paths(lib, helpers):
    rng = np.random.default_rng(1)
    v = random_gates(2, rng); perms = brickwall_perms(6, 2)
    rc, f = lib.brickwall_target(mgcu.ufunc_address(helpers.mgt_failing_ufunc), None, v, perms, 6)
    assert rc == -2
    t = lib.target_brickwall(random_gates(2, rng), brickwall_perms(8, 2), 8)
    try:
        rc, f = lib.brickwall_target(lib.mg_target_apply, t, v, perms, 6)   # 8-qubit target, 6-qubit circuit
        assert rc < 0
    finally:
        lib.target_free(t)
    # the library is still usable afterwards
    rc, f = lib.brickwall_target(mgcu.ufunc_address(helpers.mgt_hash_ufunc), None, v, perms, 6)
    assert rc == 0


def test_algebra_on_gpu(lib, oracle):
    rng = np.random.default_rng(31)
    for _ in range(4):
        u = random_gates(1, rng, unitary=True)[0]
        eta = 0.2 * rng.standard_normal(8)
        assert udist(lib.retract(u, eta), oracle.mg_retract(u, eta)) < 1e-13
    n = 40
    A = rng.standard_normal((n, n)); H = A + A.T
    g = rng.standard_normal(n)
    for radius in [0.01, 0.5, 50.0]:
        z1, b1 = lib.truncated_cg(g, H, radius, 2 * n)
        z2, b2 = oracle.truncated_cg(g, H, radius, 2 * n)
        assert b1 == b2 and udist(z1, z2) < 1e-10


def _structured_gates(n, rng):
    """gates whose blocks are drawn from every structure the target sweep specialises:
    identity, swap, diag(1,-1), diag(1,a), diagonal, anti-diagonal, real-or-imaginary, general,
    symmetric hop"""
    def block(kind):
        z = crandn((2, 2), rng)
        if kind == 0: return np.eye(2)
        if kind == 1: return np.array([[0, 1], [1, 0]], complex)
        if kind == 2: return np.diag([1, -1]).astype(complex)
        if kind == 3: return np.diag([1, z[1, 1]])
        if kind == 4: return np.diag([z[0, 0], z[1, 1]])
        if kind == 5: return np.array([[0, z[0, 1]], [z[1, 0], 0]])
        if kind == 6:
            r = rng.standard_normal((2, 2))
            return np.where(rng.random((2, 2)) < 0.5, r + 0j, 1j * r)
        if kind == 8:   # symmetric hop [[c, i s], [i s, c]] (its own kernel path)
            th = rng.uniform(-np.pi, np.pi)
            return np.array([[np.cos(th), 1j * np.sin(th)], [1j * np.sin(th), np.cos(th)]])
        return z
    out = np.zeros((n, 8), complex)
    for g in range(n):
        out[g, :4] = block(rng.integers(9)).reshape(4)
        out[g, 4:] = block(rng.integers(9)).reshape(4)
    return out


@pytest.mark.parametrize("prec,tol", [(mgcu.PREC_FP64, 1e-12), (mgcu.PREC_MIXED, 1e-12), (mgcu.PREC_FP32, 1e-4)])
@pytest.mark.parametrize("L,tile_bits", [(8, 0), (10, 6)])
def test_structured_target_blocks_vs_oracle(lib, oracle, prec, tol, L, tile_bits):
    rng = np.random.default_rng(L + tile_bits)
    ng = 120
    gates = _structured_gates(ng, rng)
    wires = np.array([rng.choice(L, 2, replace=False) for _ in range(ng)], np.int32)
    nl = 3
    v = random_gates(nl, rng, unitary=True)
    perms = brickwall_perms(L, nl, rng)
    t = lib.target_circuit(gates, wires, L)
    lib.set_precision(prec)
    lib.set_option(mgcu.OPT_TILE_BITS, tile_bits)
    try:
        rc, f, dv = lib.brickwall_target_and_gradient(lib.mg_target_apply, t, v, perms, L)
    finally:
        lib.set_precision(mgcu.PREC_FP64)
        lib.set_option(mgcu.OPT_TILE_BITS, 0)
        lib.target_free(t)
    assert rc == 0
    f_o, dv_o = oracle.brickwall_target_and_gradient(oracle.Target("circuit", L, gates=gates, wires=wires), v, perms, L)
    scale = max(1.0, abs(f_o))
    assert abs(f - f_o) < tol * scale
    assert np.max(np.abs(dv - dv_o)) < tol * max(1.0, np.max(np.abs(dv_o)))


def test_hubbard_target_vs_oracle(lib, oracle):
    import targets as T
    rng = np.random.default_rng(6)
    L = 8
    g, w, _ = T.hubbard_trotter_circuit(L // 2, 1.0, 4.0, 0.25, 8)
    v = T.near_identity_brickwall(4, rng)
    perms = T.brickwall_perms(L, 4)
    t = lib.target_circuit(g, w, L)
    try:
        rc, f, dv, h = lib.brickwall_target_gradient_hessian(lib.mg_target_apply, t, v, perms, L)
    finally:
        lib.target_free(t)
    assert rc == 0
    f_o, dv_o, h_o = oracle.brickwall_target_gradient_hessian(oracle.Target("circuit", L, gates=g, wires=w), v, perms, L)
    assert abs(f - f_o) < 1e-12 * abs(f_o) and udist(dv, dv_o) < 1e-11 and udist(h, h_o) < 1e-11


@pytest.mark.parametrize("L,tile_bits,threads,prec", [(10, 0, 0, mgcu.PREC_FP64), (12, 0, 0, mgcu.PREC_MIXED),
                                                      (12, 9, 0, mgcu.PREC_FP64), (14, 12, 0, mgcu.PREC_MIXED),
                                                      (14, 12, 128, mgcu.PREC_FP64), (14, 10, 0, mgcu.PREC_FP32),
                                                      (14, 0, 0, mgcu.PREC_FP32), (14, 13, 0, mgcu.PREC_MIXED),
                                                      (14, 13, 512, mgcu.PREC_MIXED), (14, 13, 512, mgcu.PREC_FP64),
                                                      (14, 12, 512, mgcu.PREC_MIXED), (12, 0, 512, mgcu.PREC_FP64),
                                                      (14, 12, 128, mgcu.PREC_MIXED), (14, 0, 128, mgcu.PREC_FP32),
                                                      (16, 12, 128, mgcu.PREC_MIXED)])
def test_target_sweep_tiles_vs_oracle(lib, oracle, L, tile_bits, threads, prec):
    """the target-sweep kernel with 1, 2, 4 and 8 quartets per thread, one or several
    tiles per pass and structured and general gates (also on the dropped qubit), against
    the oracle"""
    rng = np.random.default_rng(100 + L + tile_bits + threads)
    ng = 150
    gates = np.concatenate([_structured_gates(ng // 2, rng), random_gates(ng - ng // 2, rng, unitary=True)])
    rng.shuffle(gates)
    wires = np.array([rng.choice(L, 2, replace=False) for _ in range(ng)], np.int32)
    for i in range(0, ng, 7):
        wires[i] = (rng.integers(L - 1), L - 1)
        if i + 3 < ng:
            wires[i + 3] = (L - 1, rng.integers(L - 1))
    nl = 3
    v = random_gates(nl, rng, unitary=True)
    perms = brickwall_perms(L, nl, rng)
    cols = (0, 96)
    t = lib.target_circuit(gates, wires, L)
    lib.set_precision(prec)
    lib.set_option(mgcu.OPT_TILE_BITS, tile_bits)
    lib.set_option(mgcu.OPT_THREADS, min(threads, 256))
    lib.set_option(mgcu.OPT_TARGET_THREADS, threads)
    try:
        rc, f, dv = lib.brickwall_columns(lib.mg_target_apply, t, v, perms, L, *cols)
    finally:
        lib.set_option(mgcu.OPT_TILE_BITS, 0)
        lib.set_option(mgcu.OPT_THREADS, 0)
        lib.set_option(mgcu.OPT_TARGET_THREADS, 0)
        lib.set_precision(mgcu.PREC_FP64)
        lib.target_free(t)
    assert rc == 0
    tol = 1e-4 if prec == mgcu.PREC_FP32 else 1e-12
    f_o, dv_o = oracle.brickwall_target_and_gradient(oracle.Target("circuit", L, gates=gates, wires=wires), v, perms, L, col_range=cols)
    sf, sg = max(1.0, abs(f_o)), max(1.0, np.max(np.abs(dv_o)))
    assert abs(f - f_o) < tol * sf and np.max(np.abs(dv - dv_o)) < tol * sg


def _fswap_circuit(L, n, rng, paired=True):
    """random matchgates with fermionic swaps inserted in pairs on the same wires (the
    qubit order is restored) or, with paired=False, one unpaired fermionic swap"""
    fs = np.array([0, 1, 1, 0, 1, 0, 0, -1], complex)
    gates, wires = [], []
    while len(gates) < n:
        a = rng.choice(L, 2, replace=False)
        if rng.random() < 0.3:
            gates.append(fs); wires.append(a)
            for _ in range(3):
                gates.append(random_gates(1, rng, unitary=True)[0]); wires.append(rng.choice(L, 2, replace=False))
            gates.append(fs); wires.append(a[::-1] if rng.random() < 0.5 else a)
        else:
            gates.append(random_gates(1, rng, unitary=True)[0]); wires.append(a)
    if not paired:
        gates.insert(n // 2, fs); wires.insert(n // 2, np.array([0, L - 1]))
    return np.array(gates), np.array(wires, np.int32)


@pytest.mark.parametrize("L,prec,paired,tile_bits", [(10, mgcu.PREC_FP64, True, 0), (12, mgcu.PREC_MIXED, True, 0),
                                                     (12, mgcu.PREC_FP64, True, 9), (12, mgcu.PREC_FP64, False, 0),
                                                     (14, mgcu.PREC_MIXED, True, 12), (14, mgcu.PREC_FP32, True, 0)])
def test_fswap_relabelling_vs_oracle(lib, oracle, L, prec, paired, tile_bits):
    """targets with fermionic swaps: the sweep removes paired swaps by relabelling wires
    and carries Jordan-Wigner strings on the gates in between (also through the dropped
    qubit, across tiles and passes); unpaired swaps are kept as gates"""
    rng = np.random.default_rng(200 + L + tile_bits)
    gates, wires = _fswap_circuit(L, 120, rng, paired)
    nl = 3
    v = random_gates(nl, rng, unitary=True)
    perms = brickwall_perms(L, nl, rng)
    cols = (0, 96)
    t = lib.target_circuit(gates, wires, L)
    lib.set_precision(prec)
    lib.set_option(mgcu.OPT_TILE_BITS, tile_bits)
    try:
        rc, f, dv = lib.brickwall_columns(lib.mg_target_apply, t, v, perms, L, *cols)
    finally:
        lib.set_option(mgcu.OPT_TILE_BITS, 0)
        lib.set_precision(mgcu.PREC_FP64)
        lib.target_free(t)
    assert rc == 0
    tol = 1e-4 if prec == mgcu.PREC_FP32 else 1e-12
    f_o, dv_o = oracle.brickwall_target_and_gradient(oracle.Target("circuit", L, gates=gates, wires=wires), v, perms, L, col_range=cols)
    sf, sg = max(1.0, abs(f_o)), max(1.0, np.max(np.abs(dv_o)))
    assert abs(f - f_o) < tol * sf and np.max(np.abs(dv - dv_o)) < tol * sg


@pytest.mark.parametrize("L,prec,tile_bits,cols", [(12, mgcu.PREC_FP64, 0, (0, 96)), (14, mgcu.PREC_MIXED, 0, (3, 70)),
                                                   (14, mgcu.PREC_FP64, 12, (5, 7)), (14, mgcu.PREC_FP32, 0, (0, 64)),
                                                   (12, mgcu.PREC_MIXED, 9, (1, 50))])
def test_two_columns_per_block_vs_oracle(lib, oracle, L, prec, tile_bits, cols):
    """the target sweep with two basis columns of equal parity per block (and single
    columns outside whole groups of four), fermionic swaps and structured gates"""
    rng = np.random.default_rng(400 + L + tile_bits)
    g1, w1 = _fswap_circuit(L, 60, rng)
    g2 = np.concatenate([_structured_gates(30, rng), random_gates(30, rng, unitary=True)])
    w2 = np.array([rng.choice(L, 2, replace=False) for _ in range(60)], np.int32)
    gates, wires = np.concatenate([g1, g2]), np.concatenate([w1, w2])
    v = random_gates(3, rng, unitary=True)
    perms = brickwall_perms(L, 3, rng)
    t = lib.target_circuit(gates, wires, L)
    lib.set_precision(prec)
    lib.set_option(mgcu.OPT_TILE_BITS, tile_bits)
    lib.set_option(mgcu.OPT_TARGET_COLUMNS, 2)
    try:
        rc, f, dv = lib.brickwall_columns(lib.mg_target_apply, t, v, perms, L, *cols)
    finally:
        lib.set_option(mgcu.OPT_TARGET_COLUMNS, 0)
        lib.set_option(mgcu.OPT_TILE_BITS, 0)
        lib.set_precision(mgcu.PREC_FP64)
        lib.target_free(t)
    assert rc == 0
    tol = 1e-4 if prec == mgcu.PREC_FP32 else 1e-12
    f_o, dv_o = oracle.brickwall_target_and_gradient(oracle.Target("circuit", L, gates=gates, wires=wires), v, perms, L, col_range=cols)
    sf, sg = max(1.0, abs(f_o)), max(1.0, np.max(np.abs(dv_o)))
    assert abs(f - f_o) < tol * sf and np.max(np.abs(dv - dv_o)) < tol * sg


def test_hubbard_target_constructor_vs_oracle(lib, oracle):
    """mg_target_hubbard (fourth-order Suzuki circuit built by the library) as a GPU target"""
    L = 8
    g, w = lib.hubbard_trotter_circuit(L // 2, 1.0, 4.0, 0.25, 3, 4)
    t = lib.lib.mg_target_hubbard(L // 2, 1.0, 4.0, 0.25, 3, 4)
    assert t
    rng = np.random.default_rng(17)
    v = random_gates(3, rng, unitary=True)
    perms = brickwall_perms(L, 3, rng)
    try:
        rc, f, dv = lib.brickwall_target_and_gradient(lib.mg_target_apply, t, v, perms, L)
    finally:
        lib.target_free(t)
    assert rc == 0
    f_o, dv_o = oracle.brickwall_target_and_gradient(oracle.Target("circuit", L, gates=g, wires=w), v, perms, L)
    assert abs(f - f_o) < 1e-12 * max(1, abs(f_o)) and udist(dv, dv_o) < 1e-12 * max(1, np.max(np.abs(dv_o)))


@pytest.mark.parametrize("prec", [mgcu.PREC_FP64, mgcu.PREC_MIXED])
def test_resident_target_columns(lib, oracle, prec):
    """target columns kept resident on the GPU after the first evaluation: later
    evaluations with other fitted gates give the same results as sweeping the target"""
    L = 12
    rng = np.random.default_rng(55)
    gates, wires = _fswap_circuit(L, 80, rng)
    perms = brickwall_perms(L, 3, rng)
    vs = [random_gates(3, rng, unitary=True) for _ in range(3)]
    t = lib.target_circuit(gates, wires, L)
    lib.set_precision(prec)
    try:
        plain = [lib.brickwall_target_and_gradient(lib.mg_target_apply, t, v, perms, L) for v in vs]
        assert lib.target_set_resident(t, True) == 0
        res = [lib.brickwall_target_and_gradient(lib.mg_target_apply, t, v, perms, L) for v in vs]
        assert lib.target_set_resident(t, False) == 0
    finally:
        lib.set_precision(mgcu.PREC_FP64)
        lib.target_free(t)
    ot = oracle.Target("circuit", L, gates=gates, wires=wires)
    for (rc, f, dv), (rc2, f2, dv2), v in zip(plain, res, vs):
        assert rc == 0 and rc2 == 0
        assert abs(f - f2) < 1e-12 * max(1, abs(f)) and np.max(np.abs(dv - dv2)) < 1e-12 * max(1, np.max(np.abs(dv)))
        f_o, dv_o = oracle.brickwall_target_and_gradient(ot, v, perms, L)
        assert abs(f2 - f_o) < 1e-12 * max(1, abs(f_o)) and udist(dv2, dv_o) < 1e-12 * max(1, np.max(np.abs(dv_o)))
