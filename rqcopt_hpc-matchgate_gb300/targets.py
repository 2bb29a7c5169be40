"""Seeded synthetic problem instances for the benchmark configurations.

The reference measures on spinless/spinful Fermi-Hubbard Trotter circuits built by its
Python generators (benchmark_hpc/spl_hubbard1d_bench_init.py:24-118; its input files
are not shipped).  These functions build the same kinds of instances analytically,
from matchgates only, with numpy's seeded generator:

* haar_matchgates / brickwall_perms: random U(2)+U(2) gates and brickwall wirings;
* hubbard_trotter_circuit: second-order Trotter circuit of the spinful 1-D Fermi-Hubbard
  model on an open chain, sites interleaved (qubit 2s = site s spin up, 2s+1 = spin
  down), Jordan-Wigner encoded; same-spin hops between sites s, s+1 are brought next
  to each other by fermionic swaps of the two middle qubits;
* near_identity_brickwall: identity plus seeded noise, projected onto U(2)+U(2).

Gates are (n, 8) complex arrays: center block (|01>,|10>) row-major, then corner block
(|00>,|11>) row-major; a gate on wires (i, j) acts on the local index 2*bit_i + bit_j.
"""
import numpy as np


def crandn(shape, rng):
    return (rng.normal(size=shape) + 1j * rng.normal(size=shape)) / np.sqrt(2)


def _haar_u2(rng):
    q, r = np.linalg.qr(crandn((2, 2), rng))
    return q * (np.diag(r) / np.abs(np.diag(r)))


def haar_matchgates(n, rng):
    """n Haar-random U(2)+U(2) matchgates (QR of complex Gaussian blocks, phase fixed)"""
    return np.array([np.concatenate([_haar_u2(rng).reshape(4), _haar_u2(rng).reshape(4)]) for _ in range(n)])


def brickwall_perms(L, nlayers, periodic=True):
    """alternating layers: pairs (0,1),(2,3),... then (1,2),(3,4),...,(L-1,0)"""
    even = np.arange(L)
    odd = np.roll(np.arange(L), -1)
    return np.array([even if i % 2 == 0 else odd for i in range(nlayers)], dtype=np.int32)


def _polar(a):
    u, _, vh = np.linalg.svd(a)
    return u @ vh


def near_identity_brickwall(nlayers, rng, noise=1e-2):
    """identity + noise * complex Gaussian per block, projected to the nearest unitary"""
    out = np.zeros((nlayers, 8), complex)
    for i in range(nlayers):
        for b in range(2):
            out[i, 4 * b:4 * b + 4] = _polar(np.eye(2) + noise * crandn((2, 2), rng)).reshape(4)
    return out


def _gate(center, corner):
    return np.concatenate([np.asarray(center, complex).reshape(4), np.asarray(corner, complex).reshape(4)])


def onsite_gate(U, tau):
    """exp(-i U tau n_a n_b) on two modes: phase on |11>"""
    return _gate(np.eye(2), np.diag([1.0, np.exp(-1j * U * tau)]))


def hop_gate(J, tau):
    """exp(-i tau H) for H = -J (c_a^dag c_b + h.c.) on adjacent Jordan-Wigner qubits:
    exp(i J tau X) on span{|01>, |10>}"""
    c, s = np.cos(J * tau), np.sin(J * tau)
    return _gate([[c, 1j * s], [1j * s, c]], np.eye(2))


FSWAP = _gate([[0, 1], [1, 0]], np.diag([1.0, -1.0]))


def _merge(gates, wires):
    """merge consecutive gates on the same ordered wire pair (their product is a matchgate)"""
    out_g, out_w = [], []
    for g, w in zip(gates, wires):
        if out_w and tuple(out_w[-1]) == tuple(w):
            a, b = out_g[-1], g
            c = np.concatenate([(b[:4].reshape(2, 2) @ a[:4].reshape(2, 2)).reshape(4),
                                (b[4:].reshape(2, 2) @ a[4:].reshape(2, 2)).reshape(4)])
            out_g[-1] = c
        else:
            out_g.append(np.asarray(g, complex)); out_w.append(tuple(w))
    return np.array(out_g), np.array(out_w, dtype=np.int32)


def hubbard_trotter_circuit(nsites, J, U, t, nsteps):
    """Second-order Trotter circuit S(dt)^nsteps, dt = t/nsteps, for the open-chain spinful
    Fermi-Hubbard model H = -J sum_{s,sigma} (c^dag_{s,sigma} c_{s+1,sigma} + h.c.)
    + U sum_s n_{s,up} n_{s,down}, with S(dt) = A(dt/2) B(dt/2) C(dt) B(dt/2) A(dt/2) for
    A = on-site terms, B = hops on even bonds, C = hops on odd bonds.  Returns (gates,
    wires) on L = 2 * nsites qubits."""
    L = 2 * nsites
    dt = t / nsteps
    gates, wires = [], []

    def onsite(tau):
        for s in range(nsites):
            gates.append(onsite_gate(U, tau)); wires.append((2 * s, 2 * s + 1))

    def bonds(parity, tau):
        ss = [s for s in range(parity, nsites - 1, 2)]
        for s in ss:
            gates.append(FSWAP); wires.append((2 * s + 1, 2 * s + 2))
        for s in ss:
            gates.append(hop_gate(J, tau)); wires.append((2 * s, 2 * s + 1))       # spin up pair
            gates.append(hop_gate(J, tau)); wires.append((2 * s + 2, 2 * s + 3))   # spin down pair
        for s in ss:
            gates.append(FSWAP); wires.append((2 * s + 1, 2 * s + 2))

    # the trailing A(dt/2) of a step and the leading A(dt/2) of the next combine to A(dt)
    onsite(dt / 2)
    for k in range(nsteps):
        bonds(0, dt / 2)
        bonds(1, dt)
        bonds(0, dt / 2)
        onsite(dt if k < nsteps - 1 else dt / 2)
    g, w = _merge(gates, wires)
    return g, w, L


def circuit_unitary(gates, wires, L):
    """dense 2^L x 2^L matrix of a matchgate circuit (small L only; for tests)"""
    n = 1 << L
    M = np.eye(n, dtype=complex)
    for g, (i, j) in zip(gates, wires):
        G4 = np.zeros((4, 4), complex)
        G4[1:3, 1:3] = g[:4].reshape(2, 2)
        G4[0, 0], G4[0, 3], G4[3, 0], G4[3, 3] = g[4], g[5], g[6], g[7]
        T = M.reshape([2] * L + [n])
        T = np.moveaxis(T, [i, j], [0, 1]).reshape(4, -1)
        T = (G4 @ T).reshape([2, 2] + [2] * (L - 2) + [n])
        M = np.moveaxis(T, [0, 1], [i, j]).reshape(n, n)
    return M


def merge_runs(indices, coeffs):
    """neighbouring layers of the same term merged (their coefficients added)"""
    mi, mc = [], []
    for i, c in zip(indices, coeffs):
        if mi and mi[-1] == i:
            mc[-1] += c
        else:
            mi.append(i); mc.append(c)
    return mi, mc


def suzuki_rule(nterms, k):
    """Suzuki's symmetric product rule of order 2k over nterms terms, as (term index,
    coefficient) per layer with neighbouring layers of one term merged: S_2 = the terms
    forward then backward with coefficient 1/2 each, S_2k = S_2k-2 at p, p, 1-4p, p, p with
    p = 1/(4 - 4^(1/(2k-1))) (M. Suzuki, Phys. Lett. A 146, 319 (1990); the reference's
    generator, test/rqcopt_matfree/splitting_method.py:161-193)"""
    if k == 1:
        return merge_runs(list(range(nterms)) + list(range(nterms))[::-1], [0.5] * (2 * nterms))
    p = 1.0 / (4.0 - 4.0 ** (1.0 / (2 * k - 1)))
    i1, c1 = suzuki_rule(nterms, k - 1)
    return merge_runs(i1 * 5, [w * c for w in (p, p, 1 - 4 * p, p, p) for c in c1])


def spinless_hubbard_gate(J, g, tau):
    """exp(-i tau h) for the two-site term h = -J (|01><10| + |10><01|) + g |11><11| of the
    spinless Fermi-Hubbard chain (Jordan-Wigner, nearest neighbours): center block
    exp(i tau J X), corner block diag(1, exp(-i tau g))"""
    c, s = np.cos(J * tau), np.sin(J * tau)
    return _gate([[c, 1j * s], [1j * s, c]], np.diag([1.0, np.exp(-1j * g * tau)]))


def spinless_hubbard_brickwall(L, J, g, t, nsteps, order):
    """The reference's benchmark circuits (benchmark_hpc/spl_hubbard1d_bench_init.py:24-118):
    nsteps steps of the order-`order` Suzuki rule over time t for the spinless 1-D Hubbard
    model on L sites, terms = even bonds (pairs (0,1),(2,3),...) and odd bonds ((1,2),...,
    (L-1,0), periodic wiring), neighbouring layers of one term merged across steps.  Returns
    (gates [nlayers, 8], perms [nlayers, L]): one matchgate per layer on all L/2 pairs."""
    i1, c1 = suzuki_rule(2, order // 2)
    idx, cf = merge_runs(i1 * nsteps, c1 * nsteps)
    dt = t / nsteps
    gates = np.array([spinless_hubbard_gate(J, g, c * dt) for c in cf])
    even, odd = np.arange(L), np.roll(np.arange(L), -1)
    perms = np.array([even if i == 0 else odd for i in idx], dtype=np.int32)
    return gates, perms
