"""Mixed and FP32 precision against the FP64 path, and the trust-region optimiser
against the oracle's restatement of the reference's (src/trust_region.c:235-306 driven
as in src/mg_brickwall_opt.c:99-122)."""
import numpy as np
import pytest

import mgcu
import targets as T
from conftest import brickwall_perms, random_gates, rel, udist

pytestmark = pytest.mark.gpu

# stated tolerances: relative 2-norm error against the FP64 result
TOL_MIXED = 1e-9
TOL_FP32 = 1e-4


@pytest.fixture(scope="module")
def lib(mglib):
    for o in (1, 2, 3, 4):
        mglib.set_option(o, 0)
    yield mglib
    mglib.set_precision(mgcu.PREC_FP64)


def _hubbard(lib, L):
    g, w, _ = T.hubbard_trotter_circuit(L // 2, 1.0, 4.0, 0.25, 16)
    return lib.target_circuit(g, w, L)


@pytest.mark.parametrize("L,tile_bits", [(8, 0), (10, 0), (12, 0), (12, 7)])
def test_mixed_and_fp32_gradient(lib, L, tile_bits):
    rng = np.random.default_rng(L)
    nl = 5
    v = T.near_identity_brickwall(nl, rng)
    perms = T.brickwall_perms(L, nl)
    t = _hubbard(lib, L)
    lib.set_option(mgcu.OPT_TILE_BITS, tile_bits)
    try:
        out = {}
        for p in (mgcu.PREC_FP64, mgcu.PREC_MIXED, mgcu.PREC_FP32):
            lib.set_precision(p)
            rc, f, g = lib.brickwall_projected_gradient(lib.mg_target_apply, t, v, perms, L)
            rc2, f2, dv = lib.brickwall_target_and_gradient(lib.mg_target_apply, t, v, perms, L)
            assert rc == 0 and rc2 == 0
            out[p] = (f, g, dv)
    finally:
        lib.set_option(mgcu.OPT_TILE_BITS, 0)
        lib.set_precision(mgcu.PREC_FP64)
        lib.target_free(t)
    f64, g64, dv64 = out[mgcu.PREC_FP64]
    fm, gm, dvm = out[mgcu.PREC_MIXED]
    assert abs(fm - f64) / abs(f64) < TOL_MIXED
    assert rel(dvm, dv64) < TOL_MIXED
    assert rel(gm, g64) < 1e-6   # the projected gradient is small near identity: absolute 1e-9 scale
    assert np.max(np.abs(gm - g64)) < 1e-9 * np.max(np.abs(dv64))
    ff, gf, dvf = out[mgcu.PREC_FP32]
    assert abs(ff - f64) / abs(f64) < TOL_FP32 and rel(dvf, dv64) < TOL_FP32


def test_mixed_hessian(lib):
    rng = np.random.default_rng(5)
    L, nl = 8, 4
    v = random_gates(nl, rng, unitary=True)
    perms = brickwall_perms(L, nl)
    t = lib.target_brickwall(random_gates(8, rng, unitary=True), brickwall_perms(L, 8, rng), L)
    try:
        lib.set_precision(mgcu.PREC_FP64)
        rc, f, g, H = lib.brickwall_gradvec_hessmat(lib.mg_target_apply, t, v, perms, L)
        lib.set_precision(mgcu.PREC_MIXED)
        rc2, fm, gm, Hm = lib.brickwall_gradvec_hessmat(lib.mg_target_apply, t, v, perms, L)
    finally:
        lib.set_precision(mgcu.PREC_FP64)
        lib.target_free(t)
    assert rc == 0 and rc2 == 0
    assert abs(fm - f) / abs(f) < TOL_MIXED and rel(gm, g) < TOL_MIXED and rel(Hm, H) < TOL_MIXED


def test_trust_region_matches_oracle(lib, oracle):
    """10 trust-region iterations at L=8 (4 layers) against a depth-8 random matchgate
    brickwall target: every iterate's f equals the oracle's"""
    rng = np.random.default_rng(1)
    L, nl, ul = 8, 4, 8
    perms = brickwall_perms(L, nl)
    uperms = brickwall_perms(L, ul)
    ulist = random_gates(ul, rng, unitary=True)
    v0 = random_gates(nl, rng, unitary=True)
    niter = 10
    lib.set_precision(mgcu.PREC_FP64)
    t = lib.target_brickwall(ulist, uperms, L)
    try:
        f_g, fc_g, v_g = lib.optimize_brickwall(lib.mg_target_apply, t, v0, perms, L, niter)
    finally:
        lib.target_free(t)
    f_o, fc_o, v_o = oracle.rtr_brickwall(oracle.Target("brickwall", L, ulist=ulist, uperms=uperms), v0, perms, L, niter)
    assert np.max(np.abs(f_g - f_o)) < 1e-8
    assert udist(v_g, v_o) < 1e-8
    assert f_g[-1] < f_g[0]


def test_c_driver_trust_region_matches_oracle(lib, oracle, trdriver):
    """the same 10 iterations driven from C (tests/helpers/mg_test_tr_driver.c: the
    reference's optimiser glue, src/mg_brickwall_opt.c:99-122, compiled against include/ and
    linked to libmgcu.so): f_iter, f_citer and the final gates equal the oracle's"""
    import ctypes as C
    rng = np.random.default_rng(1)
    L, nl, ul = 8, 4, 8
    perms = brickwall_perms(L, nl)
    uperms = brickwall_perms(L, ul)
    ulist = random_gates(ul, rng, unitary=True)
    v0 = np.ascontiguousarray(random_gates(nl, rng, unitary=True), np.complex128)
    niter = 10
    lib.set_precision(mgcu.PREC_FP64)
    t = lib.target_brickwall(ulist, uperms, L)
    pr = np.ascontiguousarray(np.asarray(perms, np.int32).reshape(nl, L))
    rows = (C.c_void_p * nl)(*[pr[i].ctypes.data for i in range(nl)])
    f_iter = np.zeros(niter + 1)
    f_citer = np.zeros(niter + 1, np.complex128)
    vopt = np.zeros((nl, 8), np.complex128)
    try:
        rc = trdriver.mgt_optimize_brickwall_hmat(C.c_void_p(lib.mg_target_apply), C.c_void_p(t),
                                                  C.c_void_p(v0.ctypes.data), nl, L, rows, niter, C.c_void_p(f_iter.ctypes.data),
                                                  C.c_void_p(f_citer.ctypes.data), C.c_void_p(vopt.ctypes.data))
    finally:
        lib.target_free(t)
    assert rc == 0
    f_o, fc_o, v_o = oracle.rtr_brickwall(oracle.Target("brickwall", L, ulist=ulist, uperms=uperms), v0, perms, L, niter)
    assert np.max(np.abs(f_iter - f_o)) < 1e-8
    assert np.max(np.abs(f_citer - fc_o)) < 1e-8
    assert udist(vopt, v_o) < 1e-8
    assert f_iter[-1] < f_iter[0]


def test_native_trust_region_and_refinement(lib, oracle):
    """mg_optimize_brickwall: complex128 throughout matches the oracle's 10 iterations;
    float-float first with the switch to complex128 near convergence reaches the same
    iterates to 1e-9"""
    rng = np.random.default_rng(1)
    L, nl, ul = 8, 4, 8
    perms = brickwall_perms(L, nl)
    uperms = brickwall_perms(L, ul)
    ulist = random_gates(ul, rng, unitary=True)
    v0 = random_gates(nl, rng, unitary=True)
    niter = 10
    t = lib.target_brickwall(ulist, uperms, L)
    try:
        f64, p64, v64 = lib.optimize_native(t, v0, perms, L, niter)
        fmx, pmx, vmx = lib.optimize_native(t, v0, perms, L, niter, refine_gnorm=9.0)   # |grad| 12.9 -> 6.6
    finally:
        lib.set_precision(mgcu.PREC_FP64)
        lib.target_free(t)
    f_o, fc_o, v_o = oracle.rtr_brickwall(oracle.Target("brickwall", L, ulist=ulist, uperms=uperms), v0, perms, L, niter)
    assert np.all(p64 == mgcu.PREC_FP64)
    assert np.max(np.abs(f64 - f_o)) < 1e-8 and udist(v64, v_o) < 1e-8
    assert pmx[0] == mgcu.PREC_MIXED and pmx[-1] == mgcu.PREC_FP64
    assert np.max(np.abs(fmx - f_o)) < 1e-9 * np.max(np.abs(f_o)) and udist(vmx, v_o) < 1e-8


def test_native_fit_resident_columns_are_bit_identical(lib):
    """mg_optimize_brickwall keeps the target's columns on the GPU during the fit
    (MG_OPT_FIT_RESIDENT 0); sweeping the target in every evaluation instead (1) gives the
    same iterates bit for bit, in complex128 and with the float-float to complex128 switch"""
    rng = np.random.default_rng(3)
    L, nl, ul = 10, 3, 6
    perms = brickwall_perms(L, nl)
    uperms = brickwall_perms(L, ul)
    t = lib.target_brickwall(random_gates(ul, rng, unitary=True), uperms, L)
    v0 = random_gates(nl, rng, unitary=True)
    out = []
    try:
        for res in (0, 1):
            lib.set_option(mgcu.OPT_FIT_RESIDENT, res)
            out.append((lib.optimize_native(t, v0, perms, L, 6), lib.optimize_native(t, v0, perms, L, 6, refine_gnorm=5.0)))
    finally:
        lib.set_option(mgcu.OPT_FIT_RESIDENT, 0)
        lib.set_precision(mgcu.PREC_FP64)
        lib.target_free(t)
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
