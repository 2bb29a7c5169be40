"""Targets given as a host map (a caller's `linear_func`, not a GPU target): the library
calls the map once per basis column from several host threads at once, as the reference
calls it from its OpenMP threads (src/matchgate_target.c:788-795), and materialises the
columns in chunks that overlap the GPU work.  Each column is independent, so the results
must be bit-identical at any thread count; and a host brickwall map (the pattern of the
reference's benchmark drivers, benchmark_hpc/benchmark_threads.c:24-33) must give the same
trace as the same brickwall handed over as a GPU target."""
import ctypes as C

import numpy as np
import pytest

import mgcu
import targets as T
from conftest import random_gates

pytestmark = pytest.mark.gpu


class HostBrickwall(C.Structure):
    """struct mgt_brickwall of tests/helpers/mg_test_ufuncs.c"""
    _fields_ = [("gates", C.c_void_p), ("perms", C.c_void_p), ("nlayers", C.c_int)]


def host_brickwall(ul, up):
    g = np.ascontiguousarray(np.asarray(ul, np.complex128).reshape(-1, 8))
    p = np.ascontiguousarray(np.asarray(up, np.int32))
    s = HostBrickwall(g.ctypes.data, p.ctypes.data, len(g))
    return s, (g, p)


@pytest.mark.parametrize("L,nl,what", [(10, 3, "hessian"), (12, 4, "gradient")])
def test_host_map_threads_bit_identical(mglib, helpers, L, nl, what):
    lib = mglib
    lib.set_precision(mgcu.PREC_FP64)
    rng = np.random.default_rng(L + nl)
    v = random_gates(nl, rng, unitary=True)
    perms = T.brickwall_perms(L, nl)
    hashf = mgcu.ufunc_address(helpers.mgt_hash_ufunc)
    out = []
    try:
        for nt in (1, 3, 8):
            lib.set_option(mgcu.OPT_HOST_THREADS, nt)
            if what == "hessian":
                out.append(lib.brickwall_target_gradient_hessian(hashf, None, v, perms, L))
            else:
                out.append(lib.brickwall_target_and_gradient(hashf, None, v, perms, L))
    finally:
        lib.set_option(mgcu.OPT_HOST_THREADS, 0)
    for r in out:
        assert r[0] == 0, lib.last_error()
    for r in out[1:]:
        assert r[1] == out[0][1]
        for a, b in zip(r[2:], out[0][2:]):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("prec,tol", [(mgcu.PREC_FP64, 1e-12), (mgcu.PREC_MIXED, 1e-9)])
def test_host_brickwall_map_matches_gpu_target(mglib, helpers, prec, tol):
    lib = mglib
    L, nl, ul_n = 12, 4, 9
    rng = np.random.default_rng(77)
    ul = T.haar_matchgates(ul_n, rng)
    up = T.brickwall_perms(L, ul_n)
    v = T.near_identity_brickwall(nl, rng)
    perms = T.brickwall_perms(L, nl)
    hb, keep = host_brickwall(ul, up)
    t = lib.target_brickwall(ul, up, L)
    lib.set_precision(prec)
    try:
        rc1, f1, g1 = lib.brickwall_projected_gradient(mgcu.ufunc_address(helpers.mgt_brickwall_ufunc), C.addressof(hb), v, perms, L)
        rc2, f2, g2 = lib.brickwall_projected_gradient(lib.mg_target_apply, t, v, perms, L)
    finally:
        lib.set_precision(mgcu.PREC_FP64)
        lib.target_free(t)
    assert rc1 == 0 and rc2 == 0, lib.last_error()
    assert abs(f1 - f2) <= tol * abs(f2)
    assert np.linalg.norm(g1 - g2) <= tol * np.linalg.norm(g2)


def test_host_map_failure_stops_every_thread(mglib, helpers):
    """a map that fails (returns < 0) makes the call return the reference's -2"""
    lib = mglib
    rng = np.random.default_rng(5)
    v = random_gates(3, rng, unitary=True)
    lib.set_option(mgcu.OPT_HOST_THREADS, 4)
    try:
        rc, f = lib.brickwall_target(mgcu.ufunc_address(helpers.mgt_failing_ufunc), None, v, T.brickwall_perms(10, 3), 10)
    finally:
        lib.set_option(mgcu.OPT_HOST_THREADS, 0)
    assert rc == -2
