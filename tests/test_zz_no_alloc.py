"""The allocation-free entry point (mg_noalloc_brickwall_target_and_gradient) against the
regular one.  It serves callers that cannot allocate GPU memory while they run (a host
that gives all device memory to its own pool up front, or a real-time loop that cannot
take cudaMalloc's implicit synchronisation), so it works in a fixed device array.  This
file is collected last on purpose: a failure here leaves every other test already run."""
import ctypes as C

import numpy as np
import pytest

import mgcu
import targets as T
from conftest import random_gates

pytestmark = pytest.mark.gpu


def _noalloc(lib, ugates, uwires, vlist, perms, L):
    fn = lib.lib.mg_noalloc_brickwall_target_and_gradient
    ug = mgcu.gates_arr(ugates)
    uw = np.ascontiguousarray(np.asarray(uwires, np.int32).reshape(-1))
    v = mgcu.gates_arr(vlist)
    pp, rows = mgcu._perm_ptrs(perms, L)
    f = np.zeros(1, np.complex128)
    dv = np.zeros((len(v), 8), np.complex128)
    rc = fn(C.c_void_p(ug.ctypes.data), len(ug), C.c_void_p(uw.ctypes.data), C.c_void_p(v.ctypes.data), len(v), L,
            C.cast(pp, C.c_void_p), C.c_void_p(f.ctypes.data), C.c_void_p(dv.ctypes.data))
    return rc, f[0], dv


# L=4 and L=6 run one warp per block (2 and 8 quartets per gate): the strided backward
# loop and the single-warp block reduction
@pytest.mark.parametrize("L,nl,ng", [(4, 2, 10), (6, 3, 30), (8, 4, 60), (10, 5, 200)])
def test_noalloc_matches_regular_entry_point(mglib, L, nl, ng):
    lib = mglib
    lib.set_precision(mgcu.PREC_FP64)
    rng = np.random.default_rng(L * 7 + nl)
    ugates = random_gates(ng, rng, unitary=True)
    uwires = np.array([rng.choice(L, 2, replace=False) for _ in range(ng)], np.int32)
    vlist = random_gates(nl, rng, unitary=True)
    perms = T.brickwall_perms(L, nl)
    t = lib.target_circuit(ugates, uwires, L)
    try:
        rc, f_ref, dv_ref = lib.brickwall_target_and_gradient(lib.mg_target_apply, t, vlist, perms, L)
    finally:
        lib.target_free(t)
    assert rc == 0
    # two calls in a row: the second must not see the first call's leftovers
    for _ in range(2):
        rc, f, dv = _noalloc(lib, ugates, uwires, vlist, perms, L)
        assert rc == 0, lib.last_error()
        assert abs(f - f_ref) < 1e-12 * max(1.0, abs(f_ref))
        assert np.max(np.abs(dv - dv_ref)) < 1e-11


def test_noalloc_rejects_sizes_beyond_its_array(mglib):
    rng = np.random.default_rng(3)
    L = 12
    rc, f, dv = _noalloc(mglib, random_gates(4, rng), np.array([[0, 1]] * 4, np.int32), random_gates(2, rng),
                         T.brickwall_perms(L, 2), L)
    assert rc == -6
    assert "fixed workspace" in mglib.last_error()


def test_noalloc_rejects_repeated_wires(mglib):
    """a layer whose wiring repeats a qubit is rejected before anything reaches the GPU"""
    rng = np.random.default_rng(4)
    L = 8
    perms = T.brickwall_perms(L, 2).copy()
    perms[1, 7] = perms[1, 6]
    rc, f, dv = _noalloc(mglib, random_gates(4, rng), np.array([[0, 1]] * 4, np.int32), random_gates(2, rng), perms, L)
    assert rc == -6
    assert "invalid permutation of layer 1" in mglib.last_error()
