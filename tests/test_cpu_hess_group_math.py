"""The identity behind the grouped Hessian items, checked on the CPU with dense states: for
parameters shared by the gates of a block (a brickwall layer), carrying one forward-mode
state per (column, block, entry) -- it starts as the placeholder state at the block's first
gate, and at every later gate s of the block becomes G_s B + E_x F_s -- and contracting it at
every later gate with the upstream derivative gives exactly the per-layer complex Hessian
that the reference assembles from one placeholder state per gate
(src/matchgate_brickwall.c:137-260, restated by the oracle), after the same symmetrisation
of the diagonal blocks and mirroring of the lower blocks.  Conventions follow the oracle:
qubit 0 is the most significant bit, a gate on wires (i, j) maps the local index
2 bit_i + bit_j with the 4x4 matrix [[k0, 0, 0, k1], [0, c0, c1, 0], [0, c2, c3, 0],
[k2, 0, 0, k3]], and the upstream derivative is -conj(U e_b)."""
import numpy as np
import pytest

import targets as T


def _mat(g):
    c, k = g[:4], g[4:]
    return np.array([[k[0], 0, 0, k[1]], [0, c[0], c[1], 0], [0, c[2], c[3], 0], [k[2], 0, 0, k[3]]])


def _apply(M, i, j, psi, L):
    """M (4x4 on local index 2 bit_i + bit_j) applied to wires (i, j) of the 2^L vector psi"""
    t = np.moveaxis(psi.reshape((2,) * L), [i, j], [0, 1]).reshape(4, -1)
    return np.moveaxis((M @ t).reshape((2, 2) + (2,) * (L - 2)), [0, 1], [i, j]).reshape(-1)


def _unit(x):
    """E_x: the 4x4 matrix of block entry x (0-3 center, 4-7 corner), as a gate"""
    g = np.zeros(8, complex)
    g[x] = 1.0
    return _mat(g)


def _contract(i, j, L, dout, psi):
    """the 8 gate-gradient entries sum_quartets dout[r] psi[s] (oracle convention): center
    (0,0) dy y, (0,1) dy z, (1,0) dz y, (1,1) dz z; corner (0,0) dx x, (0,1) dx w, (1,0) dw x,
    (1,1) dw w"""
    d = np.moveaxis(dout.reshape((2,) * L), [i, j], [0, 1]).reshape(4, -1)
    p = np.moveaxis(psi.reshape((2,) * L), [i, j], [0, 1]).reshape(4, -1)
    x, y, z, w = 0, 1, 2, 3
    pairs = [(y, y), (y, z), (z, y), (z, z), (x, x), (x, w), (w, x), (w, w)]
    return np.array([np.sum(d[r] * p[s]) for r, s in pairs])


def _symmetrize(h, nb):
    h = h.copy()
    for i in range(nb):
        blk = h[8 * i:8 * i + 8, 8 * i:8 * i + 8]
        h[8 * i:8 * i + 8, 8 * i:8 * i + 8] = blk + blk.T
    for i in range(nb):
        for j in range(i):
            h[8 * i:8 * i + 8, 8 * j:8 * j + 8] = h[8 * j:8 * j + 8, 8 * i:8 * i + 8].T
    return h


def grouped_hessian(vlist, perms, ul, up, L):
    nl = len(vlist)
    gates = [(l, perms[l][p], perms[l][p + 1]) for l in range(nl) for p in range(0, L, 2)]
    ng = len(gates)
    n = 1 << L
    # target U column by column
    U = np.eye(n, dtype=complex)
    for l in range(len(ul)):
        for p in range(0, L, 2):
            U = np.stack([_apply(_mat(ul[l]), up[l][p], up[l][p + 1], U[:, b], L) for b in range(n)], axis=1)
    H = np.zeros((8 * nl, 8 * nl), complex)
    for b in range(n):
        F = []
        psi = np.zeros(n, complex)
        psi[b] = 1.0
        for (l, i, j) in gates:
            F.append(psi)
            psi = _apply(_mat(vlist[l]), i, j, psi, L)
        # upstream derivatives: D[k] enters gate k's backward step
        D = [None] * ng
        d = -np.conj(U[:, b])
        for k in range(ng - 1, -1, -1):
            D[k] = d
            l, i, j = gates[k]
            d = _apply(_mat(vlist[l]).T, i, j, d, L)
        for blk in range(nl):
            k0 = min(k for k in range(ng) if gates[k][0] == blk)
            for x in range(8):
                B = None
                for k in range(k0, ng):
                    l, i, j = gates[k]
                    if k > k0:
                        H[8 * blk + x, 8 * l:8 * l + 8] += _contract(i, j, L, D[k], B)
                    B = _apply(_mat(vlist[l]), i, j, B, L) if B is not None else np.zeros(n, complex)
                    if l == blk:
                        B = B + _apply(_unit(x), i, j, F[k], L)
    return _symmetrize(H, nl)


@pytest.mark.parametrize("L,nl,nu", [(4, 2, 3), (6, 3, 4)])
def test_grouped_forward_mode_equals_reference_hessian(oracle, L, nl, nu):
    rng = np.random.default_rng(40 + L)
    ul, up = T.haar_matchgates(nu, rng), T.brickwall_perms(L, nu)
    v, perms = T.haar_matchgates(nl, rng), T.brickwall_perms(L, nl)
    H = grouped_hessian(v, perms, ul, up, L)
    f_o, dv_o, h_o = oracle.brickwall_target_gradient_hessian(oracle.Target("brickwall", L, ulist=ul, uperms=up), v, perms, L)
    assert np.max(np.abs(H - h_o)) <= 1e-12 * np.max(np.abs(h_o))
