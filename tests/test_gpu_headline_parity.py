"""The benchmarked workload itself against the oracle: L=16 spinful Hubbard Trotter target
(64 second-order steps, 3336 gates, of which 1408 fermionic swaps the sweep removes by
relabelling wires, leaving gates with Jordan-Wigner strings), 5-layer periodic brickwall fit,
the same seeded instance bench.py times.  The GPU traces basis columns from the start,
middle and end of the 2^16 range (both parities in each), in complex128 and in float-float,
and each range is compared with the oracle's trace over the same columns
(reference src/matchgate_target.c:212-302, restated in oracle/mg_oracle.c).

Tolerances: complex128 1e-12 relative (f and the gradient), float-float 1e-9 relative, the
accuracy the benchmark claims for its mixed-precision value."""
import os
import sys

import numpy as np
import pytest

import mgcu

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402

pytestmark = pytest.mark.gpu

L, NLAYERS, TROTTER_STEPS = 16, 5, 64
RANGES = [(0, 16), (32760, 32776), (65520, 65536)]


@pytest.fixture(scope="module")
def headline(oracle):
    g, w, v, perms = bench.workload(L, NLAYERS, TROTTER_STEPS)
    t = oracle.Target("circuit", L, gates=g, wires=w)
    ref = [oracle.brickwall_target_and_gradient(t, v, perms, L, col_range=r) for r in RANGES]
    return g, w, v, perms, ref


def _rel(x, y):
    x, y = np.asarray(x), np.asarray(y)
    return float(np.linalg.norm(x - y) / np.linalg.norm(y))


@pytest.mark.parametrize("dense,target_threads", [(0, 0), (1, 0), (1, 128), (1, 256)])
@pytest.mark.parametrize("prec,tol", [(mgcu.PREC_FP64, 1e-12), (mgcu.PREC_MIXED, 1e-9)])
def test_headline_columns_vs_oracle(mglib, headline, prec, tol, dense, target_threads):
    """dense=0: the library's choice for this target, which conserves the Hamming weight
    (the sweep touches only amplitudes of the column's weight); dense=1: every amplitude,
    with target_threads threads per block (0: the library's choice; 128: eight quartets per
    thread, 256: four)"""
    lib = mglib
    g, w, v, perms, ref = headline
    t = lib.target_circuit(g, w, L)
    assert lib.lib.mg_target_sweep_gates(mgcu.P(t)) == 1928   # fermionic swaps relabelled away
    lib.set_precision(prec)
    lib.set_option(mgcu.OPT_TARGET_DENSE, dense)
    lib.set_option(mgcu.OPT_TARGET_THREADS, target_threads)
    try:
        for r, (f_o, dv_o) in zip(RANGES, ref):
            rc, f, dv = lib.brickwall_columns(lib.mg_target_apply, t, v, perms, L, *r)
            assert rc == 0, lib.last_error()
            assert abs(f - f_o) <= tol * abs(f_o), (r, f, f_o)
            assert _rel(dv, dv_o) <= tol, (r, _rel(dv, dv_o))
    finally:
        lib.set_option(mgcu.OPT_TARGET_THREADS, 0)
        lib.set_option(mgcu.OPT_TARGET_DENSE, 0)
        lib.set_precision(mgcu.PREC_FP64)
        lib.target_free(t)


@pytest.mark.parametrize("prec", [mgcu.PREC_FP64, mgcu.PREC_MIXED, mgcu.PREC_FP32])
def test_weight_restricted_sweep_is_bit_identical(mglib, prec):
    """the weight-restricted sweep skips only quartets of zeros: f and the gradients equal
    the full sweep's bit for bit (headline target, columns from both ends of the range)"""
    lib = mglib
    g, w, v, perms = bench.workload(L, NLAYERS, TROTTER_STEPS)
    t = lib.target_circuit(g, w, L)
    lib.set_precision(prec)
    try:
        out = []
        for dense in (0, 1):
            lib.set_option(mgcu.OPT_TARGET_DENSE, dense)
            out.append([lib.brickwall_columns(lib.mg_target_apply, t, v, perms, L, *r) for r in [(0, 40), (65500, 65536)]])
    finally:
        lib.set_option(mgcu.OPT_TARGET_DENSE, 0)
        lib.set_precision(mgcu.PREC_FP64)
        lib.target_free(t)
    for (rc0, f0, dv0), (rc1, f1, dv1) in zip(*out):
        assert rc0 == 0 and rc1 == 0
        assert f0 == f1 and np.array_equal(dv0, dv1)


@pytest.mark.parametrize("prec,tol", [(mgcu.PREC_FP64, 1e-12), (mgcu.PREC_MIXED, 1e-9)])
def test_published_workload_columns_vs_oracle(mglib, oracle, prec, tol):
    """the reference's own benchmark inputs (bench.py --config published): 601-layer
    spinless Hubbard brickwall target, 5-layer fit, on columns from both ends of the range"""
    lib = mglib
    ul, up, v, perms = bench.published_workload(L)
    t_o = oracle.Target("brickwall", L, ulist=ul, uperms=up)
    t = lib.target_brickwall(ul, up, L)
    lib.set_precision(prec)
    try:
        for r in [(0, 8), (65528, 65536)]:
            f_o, dv_o = oracle.brickwall_target_and_gradient(t_o, v, perms, L, col_range=r)
            rc, f, dv = lib.brickwall_columns(lib.mg_target_apply, t, v, perms, L, *r)
            assert rc == 0, lib.last_error()
            assert abs(f - f_o) <= tol * abs(f_o), (r, f, f_o)
            assert _rel(dv, dv_o) <= tol, (r, _rel(dv, dv_o))
    finally:
        lib.set_precision(mgcu.PREC_FP64)
        lib.target_free(t)
