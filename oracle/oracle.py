"""ctypes wrapper of the oracle (test infrastructure only).

Loads ``oracle/_build/libmgoracle.so`` (the C restatement, built by
``oracle/build_oracle.py``) and exposes numpy-facing helpers.  Gates are numpy complex128
arrays of shape (n, 8): entries 0..3 the row-major center block, 4..7 the corner
block -- the memory layout of the reference's ``struct matchgate``.  Permutations
are int32 arrays of shape (nlayers, L).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_cd = np.complex128
P = C.c_void_p


def _p(a):
    return a.ctypes.data_as(P) if a is not None else None


def lib():
    global _LIB
    if _LIB is None:
        import build_oracle as _b
        path = os.path.join(HERE, "_build", "libmgoracle.so")
        if not os.path.exists(path):
            _b.build_oracle()
        L = C.CDLL(path)
        L.orc_target_hash.restype = P
        L.orc_target_dense.restype = P
        L.orc_target_brickwall.restype = P
        L.orc_target_circuit.restype = P
        for name in ["orc_target_hash", "orc_target_dense", "orc_target_brickwall", "orc_target_circuit"]:
            getattr(L, name).argtypes = None
        L.orc_target_hash.argtypes = [C.c_int]
        L.orc_target_dense.argtypes = [P, C.c_int]
        L.orc_target_brickwall.argtypes = [P, C.c_int, P, C.c_int]
        L.orc_target_circuit.argtypes = [P, C.c_int, P, C.c_int]
        L.orc_target_free.argtypes = [P]
        L.orc_truncated_cg.restype = C.c_int
        _LIB = L
    return _LIB


import sys as _sys  # noqa: E402
if HERE not in _sys.path:
    _sys.path.insert(0, HERE)


def gates_arr(g):
    g = np.ascontiguousarray(np.asarray(g, dtype=_cd).reshape(-1, 8))
    return g


def perms_arr(p, L):
    return np.ascontiguousarray(np.asarray(p, dtype=np.int32).reshape(-1, L))


class Target:
    """Owning handle of an oracle target (the caller-supplied map U)."""

    def __init__(self, kind, L, **kw):
        self.L = L
        lb = lib()
        self._keep = []
        if kind == "hash":
            self.h = lb.orc_target_hash(L)
        elif kind == "dense":
            U = np.ascontiguousarray(kw["U"], dtype=_cd)
            self._keep.append(U)
            self.h = lb.orc_target_dense(_p(U), L)
        elif kind == "brickwall":
            ul = gates_arr(kw["ulist"])
            up = perms_arr(kw["uperms"], L)
            self._keep += [ul, up]
            self.h = lb.orc_target_brickwall(_p(ul), len(ul), _p(up), L)
        elif kind == "circuit":
            g = gates_arr(kw["gates"])
            w = np.ascontiguousarray(np.asarray(kw["wires"], dtype=np.int32).reshape(-1))
            self._keep += [g, w]
            self.h = lb.orc_target_circuit(_p(g), len(g), _p(w), L)
        else:
            raise ValueError(kind)

    def __del__(self):
        try:
            lib().orc_target_free(C.c_void_p(self.h))
        except Exception:
            pass

    def apply(self, psi):
        psi = np.ascontiguousarray(psi, dtype=_cd)
        out = np.empty_like(psi)
        sc = np.empty_like(psi)
        lib().orc_target_apply(C.c_void_p(self.h), _p(psi), _p(out), _p(sc))
        return out


# ---------------------------------------------------------------- single gates
def apply_gate(g, i, j, L, psi):
    g = gates_arr(g); psi = np.ascontiguousarray(psi, dtype=_cd); out = np.empty_like(psi)
    lib().orc_apply_gate(_p(g), i, j, L, _p(psi), _p(out))
    return out


def apply_gate_backward(g, i, j, L, psi, dpsi_out):
    g = gates_arr(g); psi = np.ascontiguousarray(psi, dtype=_cd); d = np.ascontiguousarray(dpsi_out, dtype=_cd)
    dpsi = np.empty_like(psi); dg = np.zeros((1, 8), _cd)
    lib().orc_apply_gate_backward(_p(g), i, j, L, _p(psi), _p(d), _p(dpsi), _p(dg))
    return dpsi, dg[0]


def apply_gate_array(g, i, j, L, psi_arr):
    g = gates_arr(g); a = np.ascontiguousarray(psi_arr, dtype=_cd); out = np.empty_like(a)
    lib().orc_apply_gate_array(_p(g), i, j, L, a.shape[1], _p(a), _p(out))
    return out


def apply_gate_backward_array(g, i, j, L, psi_arr, dpsi_out):
    g = gates_arr(g); a = np.ascontiguousarray(psi_arr, dtype=_cd); d = np.ascontiguousarray(dpsi_out, dtype=_cd)
    dgs = np.zeros((a.shape[1], 8), _cd)
    lib().orc_apply_gate_backward_array(_p(g), i, j, L, a.shape[1], _p(a), _p(d), _p(dgs))
    return dgs


def apply_placeholder(i, j, L, psi):
    psi = np.ascontiguousarray(psi, dtype=_cd); out = np.zeros((len(psi), 8), _cd)
    lib().orc_apply_placeholder(i, j, L, _p(psi), _p(out))
    return out


# ---------------------------------------------------------------- sweeps
def brickwall_apply(vlist, perms, L, psi):
    v = gates_arr(vlist); p = perms_arr(perms, L); psi = np.ascontiguousarray(psi, dtype=_cd); out = np.empty_like(psi)
    lib().orc_brickwall_apply(_p(v), len(v), _p(p), L, _p(psi), _p(out))
    return out


def brickwall_forward(vlist, perms, L, psi):
    v = gates_arr(vlist); p = perms_arr(perms, L); psi = np.ascontiguousarray(psi, dtype=_cd)
    ng = len(v) * (L // 2)
    cache = np.zeros((ng, 1 << L), _cd); out = np.empty_like(psi)
    lib().orc_brickwall_forward(_p(v), len(v), _p(p), L, _p(psi), _p(cache), _p(out))
    return out, cache


def brickwall_backward(vlist, perms, L, cache, dpsi_out):
    v = gates_arr(vlist); p = perms_arr(perms, L); cache = np.ascontiguousarray(cache, dtype=_cd)
    d = np.ascontiguousarray(dpsi_out, dtype=_cd); dpsi = np.empty_like(d); dv = np.zeros((len(v), 8), _cd)
    lib().orc_brickwall_backward(_p(v), len(v), _p(p), L, _p(cache), _p(d), _p(dpsi), _p(dv))
    return dpsi, dv


def brickwall_backward_hessian(vlist, perms, L, cache, dpsi_out, ti=False):
    v = gates_arr(vlist); p = perms_arr(perms, L); cache = np.ascontiguousarray(cache, dtype=_cd)
    d = np.ascontiguousarray(dpsi_out, dtype=_cd); dpsi = np.empty_like(d); dv = np.zeros((len(v), 8), _cd)
    m = 8 * len(v); hess = np.zeros((m, m), _cd)
    lib().orc_brickwall_backward_hessian(_p(v), len(v), _p(p), L, int(ti), _p(cache), _p(d), _p(dpsi), _p(dv), _p(hess))
    return dpsi, dv, hess


def circuit_apply(gates, wires, L, psi):
    g = gates_arr(gates); w = np.ascontiguousarray(np.asarray(wires, np.int32).reshape(-1))
    psi = np.ascontiguousarray(psi, dtype=_cd); out = np.empty_like(psi)
    lib().orc_circuit_apply(_p(g), len(g), _p(w), L, _p(psi), _p(out))
    return out


# ---------------------------------------------------------------- traces
def _cols(col_range):
    return (C.c_long(col_range[0]), C.c_long(col_range[1])) if col_range else (C.c_long(0), C.c_long(-1))


def circuit_target(t, gates, wires, L, nthreads=0, col_range=None):
    g = gates_arr(gates); w = np.ascontiguousarray(np.asarray(wires, np.int32).reshape(-1)); f = np.zeros(1, _cd)
    lib().orc_circuit_target(C.c_void_p(t.h), _p(g), len(g), _p(w), L, nthreads, *_cols(col_range), _p(f))
    return f[0]


def circuit_target_and_gradient(t, gates, wires, L, nthreads=0, col_range=None):
    g = gates_arr(gates); w = np.ascontiguousarray(np.asarray(wires, np.int32).reshape(-1))
    f = np.zeros(1, _cd); dg = np.zeros((len(g), 8), _cd)
    lib().orc_circuit_target_and_gradient(C.c_void_p(t.h), _p(g), len(g), _p(w), L, nthreads, *_cols(col_range), _p(f), _p(dg))
    return f[0], dg


def circuit_target_gradient_hessian(t, gates, wires, L, nthreads=0, col_range=None):
    g = gates_arr(gates); w = np.ascontiguousarray(np.asarray(wires, np.int32).reshape(-1))
    f = np.zeros(1, _cd); dg = np.zeros((len(g), 8), _cd); m = 8 * len(g); h = np.zeros((m, m), _cd)
    lib().orc_circuit_target_gradient_hessian(C.c_void_p(t.h), _p(g), len(g), _p(w), L, nthreads, *_cols(col_range), _p(f), _p(dg), _p(h))
    return f[0], dg, h


def brickwall_target(t, vlist, perms, L, nthreads=0, col_range=None):
    v = gates_arr(vlist); p = perms_arr(perms, L); f = np.zeros(1, _cd)
    lib().orc_brickwall_target(C.c_void_p(t.h), _p(v), len(v), _p(p), L, nthreads, *_cols(col_range), _p(f))
    return f[0]


def brickwall_target_and_gradient(t, vlist, perms, L, nthreads=0, col_range=None):
    v = gates_arr(vlist); p = perms_arr(perms, L); f = np.zeros(1, _cd); dv = np.zeros((len(v), 8), _cd)
    lib().orc_brickwall_target_and_gradient(C.c_void_p(t.h), _p(v), len(v), _p(p), L, nthreads, *_cols(col_range), _p(f), _p(dv))
    return f[0], dv


def brickwall_target_gradient_hessian(t, vlist, perms, L, ti=False, nthreads=0, col_range=None):
    v = gates_arr(vlist); p = perms_arr(perms, L); f = np.zeros(1, _cd); dv = np.zeros((len(v), 8), _cd)
    m = 8 * len(v); h = np.zeros((m, m), _cd)
    lib().orc_brickwall_target_gradient_hessian(C.c_void_p(t.h), _p(v), len(v), _p(p), L, int(ti), nthreads, *_cols(col_range), _p(f), _p(dv), _p(h))
    return f[0], dv, h


def brickwall_projected_gradient(t, vlist, perms, L, nthreads=0, col_range=None):
    v = gates_arr(vlist); p = perms_arr(perms, L); f = np.zeros(1, _cd); g = np.zeros(8 * len(v))
    lib().orc_brickwall_projected_gradient(C.c_void_p(t.h), _p(v), len(v), _p(p), L, nthreads, *_cols(col_range), _p(f), _p(g))
    return f[0], g


def brickwall_gradvec_hessmat(t, vlist, perms, L, ti=False, nthreads=0):
    v = gates_arr(vlist); p = perms_arr(perms, L); f = np.zeros(1, _cd); m = 8 * len(v)
    g = np.zeros(m); H = np.zeros((m, m))
    lib().orc_brickwall_gradvec_hessmat(C.c_void_p(t.h), _p(v), len(v), _p(p), L, int(ti), nthreads, _p(f), _p(g), _p(H))
    return f[0], g, H


# ---------------------------------------------------------------- algebra / TR
def _mg1(fn, *gs):
    gs = [gates_arr(g) for g in gs]
    out = np.zeros((1, 8), _cd)
    getattr(lib(), fn)(*[_p(g) for g in gs], _p(out))
    return out[0]


def mg_multiply(a, b):
    return _mg1("orc_mg_multiply", a, b)


def mg_project_tangent(u, z):
    return _mg1("orc_mg_project_tangent", u, z)


def mg_polar(a):
    return _mg1("orc_mg_polar", a)


def mg_real_to_tangent(r, v):
    r = np.ascontiguousarray(r, dtype=np.float64); v = gates_arr(v); out = np.zeros((1, 8), _cd)
    lib().orc_mg_real_to_tangent(_p(r), _p(v), _p(out))
    return out[0]


def mg_tangent_to_real(v, z):
    v = gates_arr(v); z = gates_arr(z); r = np.zeros(8)
    lib().orc_mg_tangent_to_real(_p(v), _p(z), _p(r))
    return r


def mg_retract(u, eta):
    u = gates_arr(u); eta = np.ascontiguousarray(eta, dtype=np.float64); out = np.zeros((1, 8), _cd)
    lib().orc_mg_retract(_p(u), _p(eta), _p(out))
    return out[0]


def truncated_cg(grad, hess, radius, maxiter, abstol=1e-8, reltol=1e-6):
    g = np.ascontiguousarray(grad, np.float64); h = np.ascontiguousarray(hess, np.float64); z = np.zeros_like(g)
    onb = lib().orc_truncated_cg(_p(g), _p(h), len(g), C.c_double(radius), maxiter, C.c_double(abstol), C.c_double(reltol), _p(z))
    return z, bool(onb)


def rtr_brickwall(t, vlist0, perms, L, niter, ti=False, nthreads=0, tcg_maxiter=None,
                  rho_trust=0.125, radius_init=0.01, maxradius=0.1):
    v = gates_arr(vlist0); p = perms_arr(perms, L); nl = len(v)
    if tcg_maxiter is None:
        tcg_maxiter = 2 * 16 * nl   # the drivers pass n = 16*nlayers to set_rtr_default_params
    fi = np.zeros(niter + 1); fc = np.zeros(niter + 1, _cd); vo = np.zeros_like(v)
    lib().orc_rtr_brickwall(C.c_void_p(t.h), _p(v), nl, _p(p), L, int(ti), nthreads, niter, tcg_maxiter,
                            C.c_double(rho_trust), C.c_double(radius_init), C.c_double(maxradius), _p(fi), _p(fc), _p(vo))
    return fi, fc, vo
