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


def test_spinless_hubbard_brickwall_matches_generator_conventions():
    """the published benchmark's circuits: 5 layers (order 2, 2 steps) and 601 layers (order 6,
    12 steps); each layer gate is expm(-i tau h) of the two-site term with its blocks taken in
    struct matchgate order (center on |01>,|10>, corner on |00>,|11>)"""
    import numpy as np
    from scipy.linalg import expm
    import targets as T
    v, p = T.spinless_hubbard_brickwall(16, 1.0, 1.5, 1.0, 2, 2)
    u, up = T.spinless_hubbard_brickwall(16, 1.0, 1.5, 1.0, 12, 6)
    assert len(v) == 5 and len(u) == 601 and up.shape == (601, 16)
    assert [int(x[0]) for x in p] == [0, 1, 0, 1, 0] and list(p[1]) == list(range(1, 16)) + [0]
    _, cf = T.suzuki_rule(2, 1)
    assert np.allclose(cf, [0.5, 1.0, 0.5])
    n = np.array([[0, 0], [0, 1]]); a = np.array([[0, 1], [0, 0]])
    h = -1.0 * (np.kron(a.T, a) + np.kron(a, a.T)) + 1.5 * np.kron(n, n)
    for tau in (0.25, -0.3, 0.5):
        X = expm(-1j * tau * h)
        gate = T.spinless_hubbard_gate(1.0, 1.5, tau)
        assert np.allclose(gate[:4].reshape(2, 2), X[1:3, 1:3], atol=1e-15)
        assert np.allclose(gate[4:].reshape(2, 2), X[np.ix_([0, 3], [0, 3])], atol=1e-15)
    # coefficients of one order-6 step sum to 1 per term
    i6, c6 = T.suzuki_rule(2, 3)
    assert len(i6) == 51
    assert abs(sum(c for i, c in zip(i6, c6) if i == 0) - 1) < 1e-13 and abs(sum(c for i, c in zip(i6, c6) if i == 1) - 1) < 1e-13


@pytest.mark.parametrize("L,nsteps,order", [(16, 12, 6), (16, 2, 2), (8, 3, 4), (6, 1, 2)])
def test_spinless_brickwall_matches_python_construction(mglib, L, nsteps, order):
    """the library's spinless brickwall (the published benchmark's target: L=16, 12 steps of
    order 6 = 601 layers; its fit: 2 steps of order 2 = 5 layers) equals targets.py's layer by
    layer"""
    u, pm = mglib.spinless_hubbard_brickwall(L, 1.0, 1.5, 1.0, nsteps, order)
    u2, pm2 = T.spinless_hubbard_brickwall(L, 1.0, 1.5, 1.0, nsteps, order)
    assert u.shape == u2.shape and np.array_equal(pm, pm2)
    assert np.max(np.abs(u - u2)) < 1e-14
    if (L, nsteps, order) == (16, 12, 6):
        assert len(u) == 601
    if (L, nsteps, order) == (16, 2, 2):
        assert len(u) == 5


def test_spinless_brickwall_bad_arguments(mglib):
    for args in [(5, 1.0, 1.5, 1.0, 2, 2), (16, 1.0, 1.5, 1.0, 0, 2), (16, 1.0, 1.5, 1.0, 2, 3)]:
        assert mglib.lib.mg_spinless_hubbard_brickwall(*args, None, None, 0) < 0


@pytest.mark.parametrize("order", [2, 4, 6])
def test_spinless_brickwall_orders_approach_exact_evolution(mglib, order):
    """the spinless brickwall's layers are exp(-i tau h) on every bond of the ring, h =
    -J (|01><10| + |10><01|) + g |11><11| (the two-qubit operator the layers exponentiate, the
    periodic bond included as is); its error against exp(-i H t), H the sum of h over all
    bonds, falls as h^order when the steps double"""
    L, J, g, t = 6, 1.0, 1.5, 0.6
    h = np.zeros((4, 4), complex)
    h[1, 2] = h[2, 1] = -J
    h[3, 3] = g
    n = 1 << L
    H = np.zeros((n, n), complex)
    for i in range(L):
        j = (i + 1) % L
        for a in range(n):
            bi, bj = (a >> (L - 1 - i)) & 1, (a >> (L - 1 - j)) & 1
            for oi in (0, 1):
                for oj in (0, 1):
                    v = h[2 * oi + oj, 2 * bi + bj]
                    if v != 0:
                        b2 = a & ~(1 << (L - 1 - i)) & ~(1 << (L - 1 - j)) | (oi << (L - 1 - i)) | (oj << (L - 1 - j))
                        H[b2, a] += v
    Uex = scipy.linalg.expm(-1j * t * H)
    e = []
    for nsteps in (2, 4):
        u, pm = mglib.spinless_hubbard_brickwall(L, J, g, t, nsteps, order)
        gates = np.array([u[l] for l in range(len(u)) for _ in range(L // 2)])
        wires = np.array([[pm[l][2 * p], pm[l][2 * p + 1]] for l in range(len(u)) for p in range(L // 2)], np.int32)
        e.append(np.linalg.norm(T.circuit_unitary(gates, wires, L) - Uex, 2))
    assert 0.6 * 2 ** order < e[0] / e[1] < 1.5 * 2 ** order, (order, e)
