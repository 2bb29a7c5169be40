"""Target construction on the host (mg_hubbard_trotter_circuit): the second-order circuit
equals the seeded benchmark instance of targets.py gate by gate, and higher Suzuki orders
approach exp(-i H t) of the spinful Fermi-Hubbard chain built densely here."""
import numpy as np
import pytest
import scipy.linalg

import targets as T


def _hubbard_dense(nsites, J, U):
    """H = -J sum_{s, spin} (c+_{s} c_{s+1} + h.c.) + U sum_s n_up n_down, modes 2s + spin,
    Jordan-Wigner with qubit 0 the most significant bit, |1> = occupied"""
    L = 2 * nsites
    a = np.array([[0, 1], [0, 0]], complex)
    Z = np.diag([1.0, -1.0]).astype(complex)
    I2 = np.eye(2, dtype=complex)

    def ann(m):
        ops = [Z] * m + [a] + [I2] * (L - m - 1)
        out = ops[0]
        for o in ops[1:]:
            out = np.kron(out, o)
        return out
    c = [ann(m) for m in range(L)]
    H = np.zeros((1 << L, 1 << L), complex)
    for s in range(nsites - 1):
        for spin in (0, 1):
            m, mp = 2 * s + spin, 2 * s + 2 + spin
            hop = c[m].conj().T @ c[mp]
            H += -J * (hop + hop.conj().T)
    for s in range(nsites):
        H += U * (c[2 * s].conj().T @ c[2 * s]) @ (c[2 * s + 1].conj().T @ c[2 * s + 1])
    return H


def test_second_order_matches_benchmark_instance(mglib):
    for nsites, nsteps in [(3, 5), (8, 64)]:
        g, w = mglib.hubbard_trotter_circuit(nsites, 1.0, 4.0, 0.25, nsteps, 2)
        g2, w2, _ = T.hubbard_trotter_circuit(nsites, 1.0, 4.0, 0.25, nsteps)
        assert g.shape == g2.shape and np.array_equal(w, w2)
        assert np.max(np.abs(g - g2)) < 1e-14


@pytest.mark.parametrize("nsites", [2, 3])
def test_suzuki_orders_approach_exact_evolution(mglib, nsites):
    """the error against exp(-i H t) falls as h^order when the steps double"""
    J, U, t = 1.0, 4.0, 0.5
    L = 2 * nsites
    Uex = scipy.linalg.expm(-1j * t * _hubbard_dense(nsites, J, U))
    for order in (2, 4, 6):
        e = []
        for nsteps in (4, 8):
            g, w = mglib.hubbard_trotter_circuit(nsites, J, U, t, nsteps, order)
            e.append(np.linalg.norm(T.circuit_unitary(g, w, L) - Uex, 2))
        assert 0.7 * 2 ** order < e[0] / e[1] < 1.4 * 2 ** order, (order, e)
    assert e[1] < 1e-8


def test_bad_arguments(mglib):
    assert mglib.lib.mg_hubbard_trotter_circuit(1, 1.0, 4.0, 0.25, 4, 2, None, None, 0) < 0
    assert mglib.lib.mg_hubbard_trotter_circuit(4, 1.0, 4.0, 0.25, 4, 3, None, None, 0) < 0
