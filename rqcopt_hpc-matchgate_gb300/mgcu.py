"""ctypes binding of the matchgate C API (the reference's matchgate_brickwall.h,
matchgate_target.h, trust_region.h, gate.h, quantum_circuit.h, matchgate.h) and of
this library's extensions (mg_gb300.h).

``MatchgateLib(path)`` binds any shared library exporting that C API: this project's
``_build/libmgcu.so``, or a build of the reference, so both can be driven through the
same C entry points with numpy arrays.  Conventions:

* a gate is a complex128 array of 8 entries (center block row-major, then corner
  block), i.e. the memory of ``struct matchgate``; lists of gates are (n, 8) arrays;
* perms are int32 arrays (nlayers, L); wires are int32 arrays (ngates, 2);
* a target map is a pair (ufunc, udata) of addresses: ``lib.target_*`` returns a
  GPU target of this library, ``ufunc_address(cfunc)`` wraps C or Python callbacks.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_LIB = os.path.join(HERE, "_build", "libmgcu.so")

PREC_FP64, PREC_MIXED, PREC_FP32 = 0, 1, 2
OPT_TILE_BITS, OPT_THREADS, OPT_CHUNK_COLUMNS, OPT_CTAS_PER_SM = 1, 2, 3, 4
OPT_TARGET_TILE_BITS, OPT_TARGET_THREADS, OPT_TARGET_COLUMNS = 5, 6, 7
OPT_TRANSLATIONAL_INVARIANCE = 8
OPT_TARGET_DENSE = 9
OPT_HOST_THREADS = 10
OPT_FIT_CACHE = 11
OPT_TARGET_TUNE = 12
OPT_HESS_GROUP = 13
OPT_FIT_RESIDENT = 14
EVAL_TARGET, EVAL_GRADIENT, EVAL_HESSIAN, EVAL_TI = 0, 1, 2, 4

P = C.c_void_p
cd = np.complex128


class StateVector(C.Structure):
    _fields_ = [("data", C.c_void_p), ("nqubits", C.c_int)]


class StateVectorArray(C.Structure):
    _fields_ = [("data", C.c_void_p), ("nqubits", C.c_int), ("nstates", C.c_int)]


class CircuitCache(C.Structure):
    _fields_ = [("psi_list", C.POINTER(StateVector)), ("nqubits", C.c_int), ("ngates", C.c_int)]


class TcgParams(C.Structure):
    _fields_ = [("maxiter", C.c_int), ("abstol", C.c_double), ("reltol", C.c_double)]


TargetFunc = C.CFUNCTYPE(C.c_double, C.POINTER(C.c_double), C.c_void_p, C.POINTER(C.c_double))
TargetGradHessFunc = C.CFUNCTYPE(C.c_double, C.POINTER(C.c_double), C.c_void_p, C.POINTER(C.c_double),
                                 C.POINTER(C.c_double), C.POINTER(C.c_double))
RetractFunc = C.CFUNCTYPE(None, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p, C.POINTER(C.c_double))
LinearFunc = C.CFUNCTYPE(C.c_int, C.POINTER(StateVector), C.c_void_p, C.POINTER(StateVector))


class RtrParams(C.Structure):
    _fields_ = [("tcg_params", TcgParams), ("rho_trust", C.c_double), ("radius_init", C.c_double),
                ("maxradius", C.c_double), ("g_func", C.c_void_p), ("g_data", C.c_void_p), ("g_iter", C.c_void_p)]


class Request(C.Structure):
    """mg_request of mg_gb300.h"""
    _fields_ = [("kind", C.c_int), ("target", C.c_void_p), ("nqubits", C.c_int), ("nlayers", C.c_int),
                ("vlist", C.c_void_p), ("perms", C.c_void_p), ("radius", C.c_double)]


REQ_TARGET, REQ_GRADIENT, REQ_HESSIAN, REQ_TRSTEP = 0, 1, 2, 3


def _p(a):
    return a.ctypes.data_as(P) if a is not None else None


def gates_arr(g):
    return np.ascontiguousarray(np.asarray(g, dtype=cd).reshape(-1, 8))


def _sv(a, L):
    return StateVector(a.ctypes.data, L)


def _perm_ptrs(perms, L):
    rows = [np.ascontiguousarray(np.asarray(p, dtype=np.int32).reshape(L)) for p in perms]
    arr = (C.c_void_p * max(len(rows), 1))(*[r.ctypes.data for r in rows])
    return arr, rows


def ufunc_address(f):
    """Address of a linear_func: a ctypes function of a loaded library or a LinearFunc."""
    return C.cast(f, C.c_void_p).value


def python_ufunc(fn):
    """Wrap fn(psi: np.ndarray) -> np.ndarray as a LinearFunc (keep the result alive)."""
    def cb(psi_p, udata, out_p):
        L = psi_p.contents.nqubits
        n = 1 << L
        psi = np.ctypeslib.as_array(C.cast(psi_p.contents.data, C.POINTER(C.c_double)), shape=(2 * n,)).view(cd)
        out = np.ctypeslib.as_array(C.cast(out_p.contents.data, C.POINTER(C.c_double)), shape=(2 * n,)).view(cd)
        out[:] = fn(psi.copy())
        return 0
    return LinearFunc(cb)


class MatchgateLib:
    """numpy-facing binding of the matchgate C API exported by ``path``."""

    def __init__(self, path=DEFAULT_LIB):
        self.path = path
        self.lib = C.CDLL(path)
        L = self.lib
        self.is_gb300 = hasattr(L, "mg_set_precision")
        if self.is_gb300:
            for name in ["mg_target_brickwall", "mg_target_circuit", "mg_target_dense", "mg_plan_brickwall"]:
                getattr(L, name).restype = P
            L.mg_target_brickwall.argtypes = [P, C.c_int, P, C.c_int]
            L.mg_target_circuit.argtypes = [P, C.c_int, P, C.c_int]
            L.mg_target_dense.argtypes = [P, C.c_int]
            L.mg_target_free.argtypes = [P]
            L.mg_target_set_resident.argtypes = [P, C.c_int]
            L.mg_target_sweep_gates.argtypes = [P]
            L.mg_target_conserves_weight.argtypes = [P]
            L.mg_batch_create.restype = P
            L.mg_batch_create.argtypes = [C.c_int, P, P, P, P, P, C.c_int]
            L.mg_batch_set_gates.argtypes = [P, C.c_int, P]
            L.mg_batch_run.argtypes = [P]
            L.mg_batch_results.argtypes = [P, C.c_int, P, P, P]
            L.mg_batch_info.argtypes = [P, C.c_int, P, P, P]
            L.mg_batch_time_ms.argtypes = [P, C.c_int, C.c_int]
            L.mg_batch_time_ms.restype = C.c_double
            L.mg_batch_free.argtypes = [P]
            L.mg_hubbard_trotter_circuit.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, P, P, C.c_int]
            L.mg_target_hubbard.restype = P
            L.mg_target_hubbard.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int]
            L.mg_spinless_hubbard_brickwall.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, P, P, C.c_int]
            L.mg_target_spinless_hubbard.restype = P
            L.mg_target_spinless_hubbard.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int]
            L.mg_optimize_brickwall.argtypes = [P, P, C.c_int, C.c_int, P, C.POINTER(RtrParams), C.c_int, C.c_double, P, P, P]
            L.mg_server_create.restype = P
            L.mg_server_create.argtypes = [C.c_size_t, C.c_int]
            L.mg_server_submit.restype = C.c_long
            L.mg_server_submit.argtypes = [P, C.POINTER(Request)]
            L.mg_server_done.argtypes = [P, C.c_long]
            L.mg_server_wait.argtypes = [P, C.c_long]
            L.mg_server_result.argtypes = [P, C.c_long, P, P, P, P, P, P, P, P]
            L.mg_server_stats.argtypes = [P, P, P, P]
            L.mg_server_free.argtypes = [P]
            L.mg_last_error.restype = C.c_char_p
            L.mg_plan_brickwall.argtypes = [P, P, P, C.c_int, C.c_int, P, C.c_int]
            L.mg_plan_set_gates.argtypes = [P, P]
            L.mg_plan_run.argtypes = [P]
            L.mg_plan_results.argtypes = [P, P, P, P, P, P]
            L.mg_plan_free.argtypes = [P]
            L.mg_plan_time_ms.argtypes = [P, C.c_int, C.c_int]
            L.mg_plan_time_ms.restype = C.c_double
            L.mg_plan_target_kernel_ms.argtypes = [P, P, P]
            L.mg_plan_target_config.argtypes = [P, P]
            L.mg_launch_count.restype = C.c_long
            L.mg_get_option.restype = C.c_long
            L.mg_set_option.argtypes = [C.c_int, C.c_long]
            L.mg_measure_fp32_peak_gflops.restype = C.c_double
            L.mg_measure_fp64_peak_gflops.restype = C.c_double
            L.mg_brickwall_target_and_gradient_columns.argtypes = [P, P, P, C.c_int, C.c_int, P, C.c_long, C.c_long, P, P]
        L.truncated_cg_hmat.restype = C.c_bool
        L.truncated_cg_hmat.argtypes = [P, P, C.c_int, C.c_double, C.POINTER(TcgParams), P]
        for name in ["uniform_distance", "uniform_distance_real"]:
            getattr(L, name).restype = C.c_double
        self.mg_target_apply = ufunc_address(L.mg_target_apply) if self.is_gb300 else None
        self._keep = []

    # ------------------------------------------------------------------ settings
    def set_precision(self, p):
        return self.lib.mg_set_precision(p)

    def set_option(self, opt, value):
        return self.lib.mg_set_option(opt, value)

    def last_error(self):
        return self.lib.mg_last_error().decode()

    def plan_target_config(self, plan):
        """the plan's target sweep: dict(kind 0 none / 1 full / 2 weight-restricted, tile_bits,
        threads, per_thread)"""
        cfg = (C.c_int * 4)()
        rc = self.lib.mg_plan_target_config(P(plan), cfg)
        if rc != 0:
            raise RuntimeError(self.last_error())
        return {"kind": cfg[0], "tile_bits": cfg[1], "threads": cfg[2], "per_thread": cfg[3]}

    def plan_target_kernel_ms(self, plan):
        """(summed ms, launches) of the target-sweep kernel in the last plan timing"""
        ms, n = C.c_double(), C.c_long()
        rc = self.lib.mg_plan_target_kernel_ms(P(plan), C.byref(ms), C.byref(n))
        if rc != 0:
            raise RuntimeError(self.last_error())
        return ms.value, n.value

    # ------------------------------------------------------------------ batches
    def batch_create(self, targets, vlists, perms_list, Ls, tune=True):
        """mg_batch_create for n brickwall fits; returns an opaque batch (keeps its inputs alive)"""
        n = len(targets)
        keep = []
        vl = [gates_arr(v) for v in vlists]
        pps = []
        for perms, L in zip(perms_list, Ls):
            pp, rows = _perm_ptrs(perms, L)
            keep.append((pp, rows))
            pps.append(C.cast(pp, P).value)
        T = (P * n)(*targets)
        V = (P * n)(*[v.ctypes.data for v in vl])
        NL = (C.c_int * n)(*[len(v) for v in vl])
        PP = (P * n)(*pps)
        LL = (C.c_int * n)(*[int(L) for L in Ls])
        b = self.lib.mg_batch_create(n, T, V, NL, PP, LL, int(bool(tune)))
        if not b:
            raise RuntimeError(self.last_error())
        return {"ptr": b, "n": n, "nlayers": [len(v) for v in vl], "keep": (keep, vl)}

    def batch_set_gates(self, batch, i, vlist):
        v = gates_arr(vlist)
        return self.lib.mg_batch_set_gates(P(batch["ptr"]), i, _p(v))

    def batch_run(self, batch):
        return self.lib.mg_batch_run(P(batch["ptr"]))

    def batch_results(self, batch, i):
        """(f, dvlist [nlayers, 8], grad_vec [8 nlayers])"""
        nl = batch["nlayers"][i]
        f = np.zeros(1, cd); dv = np.zeros((nl, 8), cd); g = np.zeros(8 * nl)
        rc = self.lib.mg_batch_results(P(batch["ptr"]), i, _p(f), _p(dv), _p(g))
        if rc != 0:
            raise RuntimeError(self.last_error())
        return f[0], dv, g

    def batch_info(self, batch, i):
        kt, npass, items = C.c_int(), C.c_int(), C.c_int()
        rc = self.lib.mg_batch_info(P(batch["ptr"]), i, C.byref(kt), C.byref(npass), C.byref(items))
        if rc != 0:
            raise RuntimeError(self.last_error())
        return kt.value, npass.value, items.value

    def batch_time_ms(self, batch, steps, flush_l2=True):
        return self.lib.mg_batch_time_ms(P(batch["ptr"]), steps, int(bool(flush_l2)))

    def batch_free(self, batch):
        self.lib.mg_batch_free(P(batch["ptr"]))
        batch["ptr"] = None

    def optimize_native(self, target, vlist0, perms, L, niter, refine_gnorm=0.0, tcg_maxiter=None,
                        rho_trust=0.125, radius_init=0.01, maxradius=0.1):
        """mg_optimize_brickwall: (f_iter [niter+1], prec_iter [niter+1], final gates)"""
        v0 = gates_arr(vlist0); nl = len(v0)
        pp, rows = _perm_ptrs(perms, L)
        prm = RtrParams()
        prm.tcg_params = TcgParams(tcg_maxiter if tcg_maxiter is not None else 2 * 16 * nl, 1e-8, 1e-6)
        prm.rho_trust, prm.radius_init, prm.maxradius = rho_trust, radius_init, maxradius
        f_iter = np.zeros(niter + 1); prec = np.zeros(niter + 1, np.int32); xf = np.zeros((nl, 8), cd)
        rc = self.lib.mg_optimize_brickwall(P(target), _p(v0), nl, L, C.cast(pp, P), C.byref(prm), niter, refine_gnorm,
                                            _p(f_iter), _p(prec), _p(xf))
        if rc != 0:
            raise RuntimeError(self.last_error())
        return f_iter, prec, xf

    def optimize_circuit_native(self, target, gates0, wires, L, niter, refine_gnorm=0.0, tcg_maxiter=None,
                                rho_trust=0.125, radius_init=0.01, maxradius=0.1):
        """mg_optimize_circuit (one parameter block per gate): (f_iter, prec_iter, final gates)"""
        g0 = gates_arr(gates0); ng = len(g0)
        w = np.ascontiguousarray(np.asarray(wires, np.int32).reshape(-1))
        prm = RtrParams()
        prm.tcg_params = TcgParams(tcg_maxiter if tcg_maxiter is not None else 2 * 8 * ng, 1e-8, 1e-6)
        prm.rho_trust, prm.radius_init, prm.maxradius = rho_trust, radius_init, maxradius
        f_iter = np.zeros(niter + 1); prec = np.zeros(niter + 1, np.int32); xf = np.zeros((ng, 8), cd)
        rc = self.lib.mg_optimize_circuit(P(target), _p(g0), ng, _p(w), L, C.byref(prm), niter, C.c_double(refine_gnorm),
                                          _p(f_iter), _p(prec), _p(xf))
        if rc != 0:
            raise RuntimeError(self.last_error())
        return f_iter, prec, xf

    # ------------------------------------------------------------------ target construction
    def hubbard_trotter_circuit(self, nsites, J, U, t, nsteps, order=2):
        """(gates [n, 8], wires [n, 2]) of the Suzuki circuit built by the library"""
        n = self.lib.mg_hubbard_trotter_circuit(nsites, J, U, t, nsteps, order, None, None, 0)
        if n < 0:
            raise RuntimeError(self.last_error())
        g = np.zeros((n, 8), cd); w = np.zeros((n, 2), np.int32)
        n2 = self.lib.mg_hubbard_trotter_circuit(nsites, J, U, t, nsteps, order, _p(g), _p(w), n)
        assert n2 == n
        return g, w

    def spinless_hubbard_brickwall(self, L, J, g, t, nsteps, order=2):
        """(ulist [n, 8], perms [n, L]) of the spinless brickwall built by the library"""
        n = self.lib.mg_spinless_hubbard_brickwall(L, J, g, t, nsteps, order, None, None, 0)
        if n < 0:
            raise RuntimeError(self.last_error())
        u = np.zeros((n, 8), cd); pm = np.zeros((n, L), np.int32)
        n2 = self.lib.mg_spinless_hubbard_brickwall(L, J, g, t, nsteps, order, _p(u), _p(pm), n)
        assert n2 == n
        return u, pm

    # ------------------------------------------------------------------ request server
    def server_create(self, budget_bytes, max_batch=256):
        s = self.lib.mg_server_create(int(budget_bytes), int(max_batch))
        if not s:
            raise RuntimeError(self.last_error())
        return s

    def server_submit(self, server, kind, target, vlist, perms, L, radius=0.0):
        v = gates_arr(vlist)
        pr = np.ascontiguousarray(np.asarray(perms, np.int32).reshape(len(v), L))
        q = Request(kind, target, L, len(v), v.ctypes.data, pr.ctypes.data, radius)
        rid = self.lib.mg_server_submit(P(server), C.byref(q))
        if rid < 0:
            raise RuntimeError(self.last_error())
        return rid

    def server_done(self, server, rid):
        return self.lib.mg_server_done(P(server), rid) == 1

    def server_result(self, server, rid, nlayers):
        """dict: status, f, grad_vec, H, vlist, radius, accepted, times (submit, start, done), step"""
        n = 8 * nlayers
        f = np.zeros(1, cd); g = np.zeros(n); H = np.zeros((n, n)); v = np.zeros((nlayers, 8), cd)
        rad = C.c_double(); acc = C.c_int(); t = np.zeros(3); step = C.c_long()
        st = self.lib.mg_server_result(P(server), rid, _p(f), _p(g), _p(H), _p(v), C.byref(rad), C.byref(acc), _p(t), C.byref(step))
        return {"status": st, "f": f[0], "grad_vec": g, "H": H, "vlist": v, "radius": rad.value, "accepted": bool(acc.value),
                "times": t, "step": step.value}

    def server_stats(self, server):
        st, bt, pk = C.c_long(), C.c_long(), C.c_size_t()
        self.lib.mg_server_stats(P(server), C.byref(st), C.byref(bt), C.byref(pk))
        return st.value, bt.value, pk.value

    def server_free(self, server):
        self.lib.mg_server_free(P(server))

    def launch_count(self):
        return self.lib.mg_launch_count()

    # ------------------------------------------------------------------ GPU targets
    def target_brickwall(self, ulist, uperms, L):
        ul = gates_arr(ulist)
        pp, rows = _perm_ptrs(uperms, L)
        h = self.lib.mg_target_brickwall(_p(ul), len(ul), C.cast(pp, P), L)
        if not h:
            raise RuntimeError("mg_target_brickwall failed: " + self.last_error())
        return h

    def target_circuit(self, gates, wires, L):
        g = gates_arr(gates)
        w = np.ascontiguousarray(np.asarray(wires, np.int32).reshape(-1))
        h = self.lib.mg_target_circuit(_p(g), len(g), _p(w), L)
        if not h:
            raise RuntimeError("mg_target_circuit failed: " + self.last_error())
        return h

    def target_dense(self, U, L):
        U = np.ascontiguousarray(U, dtype=cd)
        h = self.lib.mg_target_dense(_p(U), L)
        if not h:
            raise RuntimeError("mg_target_dense failed: " + self.last_error())
        return h

    def target_set_resident(self, h, enable=True):
        return self.lib.mg_target_set_resident(P(h), int(bool(enable)))

    def target_free(self, h):
        self.lib.mg_target_free(h)

    # ------------------------------------------------------------------ single gates (gate.h)
    def apply_matchgate(self, g, i, j, psi):
        g = gates_arr(g); psi = np.ascontiguousarray(psi, dtype=cd); L = int(np.log2(len(psi)))
        out = np.zeros_like(psi)
        a, b = _sv(psi, L), _sv(out, L)
        self.lib.apply_matchgate(_p(g), i, j, C.byref(a), C.byref(b))
        return out

    def apply_matchgate_backward(self, g, i, j, psi, dpsi_out):
        g = gates_arr(g); psi = np.ascontiguousarray(psi, dtype=cd); d = np.ascontiguousarray(dpsi_out, dtype=cd)
        L = int(np.log2(len(psi))); dpsi = np.zeros_like(psi); dg = np.zeros((1, 8), cd)
        self.lib.apply_matchgate_backward(_p(g), i, j, C.byref(_sv(psi, L)), C.byref(_sv(d, L)), C.byref(_sv(dpsi, L)), _p(dg))
        return dpsi, dg[0]

    def apply_matchgate_to_array(self, g, i, j, arr):
        g = gates_arr(g); a = np.ascontiguousarray(arr, dtype=cd); L = int(np.log2(a.shape[0])); out = np.zeros_like(a)
        x = StateVectorArray(a.ctypes.data, L, a.shape[1]); y = StateVectorArray(out.ctypes.data, L, a.shape[1])
        self.lib.apply_matchgate_to_array(_p(g), i, j, C.byref(x), C.byref(y))
        return out

    def apply_matchgate_backward_array(self, g, i, j, arr, dpsi_out):
        g = gates_arr(g); a = np.ascontiguousarray(arr, dtype=cd); d = np.ascontiguousarray(dpsi_out, dtype=cd)
        L = int(np.log2(a.shape[0])); dgs = np.zeros((a.shape[1], 8), cd)
        x = StateVectorArray(a.ctypes.data, L, a.shape[1])
        self.lib.apply_matchgate_backward_array(_p(g), i, j, C.byref(x), C.byref(_sv(d, L)), _p(dgs))
        return dgs

    def apply_placeholder(self, i, j, psi, nout=8):
        psi = np.ascontiguousarray(psi, dtype=cd); L = int(np.log2(len(psi))); out = np.zeros((len(psi), nout), cd)
        y = StateVectorArray(out.ctypes.data, L, nout)
        fn = self.lib.apply_matchgate_placeholder if nout == 8 else self.lib.apply_gate_placeholder
        fn(i, j, C.byref(_sv(psi, L)), C.byref(y))
        return out

    # ------------------------------------------------------------------ sweeps on one vector
    def _cache(self, L, ng, data=None):
        rows = np.zeros((ng, 1 << L), cd) if data is None else np.ascontiguousarray(data, dtype=cd)
        svs = (StateVector * ng)(*[StateVector(rows[k].ctypes.data, L) for k in range(ng)])
        cache = CircuitCache(C.cast(svs, C.POINTER(StateVector)), L, ng)
        return cache, rows, svs

    def brickwall_apply(self, vlist, perms, psi):
        v = gates_arr(vlist); psi = np.ascontiguousarray(psi, dtype=cd); L = int(np.log2(len(psi)))
        pp, rows = _perm_ptrs(perms, L); out = np.zeros_like(psi)
        r = self.lib.apply_matchgate_brickwall_unitary(_p(v), len(v), C.cast(pp, P), C.byref(_sv(psi, L)), C.byref(_sv(out, L)))
        assert r == 0
        return out

    def brickwall_forward(self, vlist, perms, psi):
        v = gates_arr(vlist); psi = np.ascontiguousarray(psi, dtype=cd); L = int(np.log2(len(psi)))
        pp, rows = _perm_ptrs(perms, L); out = np.zeros_like(psi)
        cache, crow, svs = self._cache(L, len(v) * (L // 2))
        r = self.lib.matchgate_brickwall_unitary_forward(_p(v), len(v), C.cast(pp, P), C.byref(_sv(psi, L)), C.byref(cache), C.byref(_sv(out, L)))
        assert r == 0
        return out, crow

    def brickwall_backward(self, vlist, perms, cache_rows, dpsi_out, hessian=False, ti=False):
        v = gates_arr(vlist); d = np.ascontiguousarray(dpsi_out, dtype=cd); L = int(np.log2(len(d)))
        pp, rows = _perm_ptrs(perms, L); dpsi = np.zeros_like(d); dv = np.zeros((len(v), 8), cd)
        cache, crow, svs = self._cache(L, len(v) * (L // 2), cache_rows)
        if not hessian:
            r = self.lib.matchgate_brickwall_unitary_backward(_p(v), len(v), C.cast(pp, P), C.byref(cache), C.byref(_sv(d, L)),
                                                             C.byref(_sv(dpsi, L)), _p(dv))
            assert r == 0
            return dpsi, dv
        m = 8 * len(v); hess = np.zeros((m, m), cd)
        fn = self.lib.matchgate_ti_brickwall_unitary_backward_hessian if ti else self.lib.matchgate_brickwall_unitary_backward_hessian
        r = fn(_p(v), len(v), C.cast(pp, P), C.byref(cache), C.byref(_sv(d, L)), C.byref(_sv(dpsi, L)), _p(dv), _p(hess))
        assert r == 0
        return dpsi, dv, hess

    def circuit_apply(self, gates, wires, psi):
        g = gates_arr(gates); w = np.ascontiguousarray(np.asarray(wires, np.int32).reshape(-1))
        psi = np.ascontiguousarray(psi, dtype=cd); L = int(np.log2(len(psi))); out = np.zeros_like(psi)
        r = self.lib.apply_quantum_matchgate_circuit(_p(g), len(g), _p(w), C.byref(_sv(psi, L)), C.byref(_sv(out, L)))
        assert r == 0
        return out

    def circuit_forward(self, gates, wires, psi):
        g = gates_arr(gates); w = np.ascontiguousarray(np.asarray(wires, np.int32).reshape(-1))
        psi = np.ascontiguousarray(psi, dtype=cd); L = int(np.log2(len(psi))); out = np.zeros_like(psi)
        cache, crow, svs = self._cache(L, len(g))
        r = self.lib.quantum_matchgate_circuit_forward(_p(g), len(g), _p(w), C.byref(_sv(psi, L)), C.byref(cache), C.byref(_sv(out, L)))
        assert r == 0
        return out, crow

    def circuit_backward(self, gates, wires, cache_rows, dpsi_out):
        g = gates_arr(gates); w = np.ascontiguousarray(np.asarray(wires, np.int32).reshape(-1))
        d = np.ascontiguousarray(dpsi_out, dtype=cd); L = int(np.log2(len(d))); dpsi = np.zeros_like(d); dg = np.zeros((len(g), 8), cd)
        cache, crow, svs = self._cache(L, len(g), cache_rows)
        r = self.lib.quantum_matchgate_circuit_backward(_p(g), len(g), _p(w), C.byref(cache), C.byref(_sv(d, L)), C.byref(_sv(dpsi, L)), _p(dg))
        assert r == 0
        return dpsi, dg

    # ------------------------------------------------------------------ traces (matchgate_target.h)
    def circuit_target(self, ufunc, udata, gates, wires, L):
        g = gates_arr(gates); w = np.ascontiguousarray(np.asarray(wires, np.int32).reshape(-1)); f = np.zeros(1, cd)
        rc = self.lib.matchgate_circuit_unitary_target(P(ufunc), P(udata), _p(g), len(g), _p(w), L, _p(f))
        return rc, f[0]

    def circuit_target_and_gradient(self, ufunc, udata, gates, wires, L):
        g = gates_arr(gates); w = np.ascontiguousarray(np.asarray(wires, np.int32).reshape(-1))
        f = np.zeros(1, cd); dg = np.zeros((len(g), 8), cd)
        rc = self.lib.matchgate_circuit_unitary_target_and_gradient(P(ufunc), P(udata), _p(g), len(g), _p(w), L, _p(f), _p(dg))
        return rc, f[0], dg

    def circuit_target_gradient_hessian(self, ufunc, udata, gates, wires, L):
        g = gates_arr(gates); w = np.ascontiguousarray(np.asarray(wires, np.int32).reshape(-1))
        f = np.zeros(1, cd); dg = np.zeros((len(g), 8), cd); m = 8 * len(g); h = np.zeros((m, m), cd)
        rc = self.lib.matchgate_circuit_unitary_target_gradient_hessian(P(ufunc), P(udata), _p(g), len(g), _p(w), L, _p(f), _p(dg), _p(h))
        return rc, f[0], dg, h

    def circuit_gradvec_hessmat(self, ufunc, udata, gates, wires, L):
        """per-gate Riemannian gradient [8 ngates] and Hessian [(8 ngates)^2]"""
        g = gates_arr(gates); w = np.ascontiguousarray(np.asarray(wires, np.int32).reshape(-1))
        f = np.zeros(1, cd); m = 8 * len(g); gv = np.zeros(m); H = np.zeros((m, m))
        rc = self.lib.matchgate_circuit_unitary_target_gradient_vector_hessian_matrix(P(ufunc), P(udata), _p(g), len(g), _p(w), L,
                                                                                     _p(f), _p(gv), _p(H))
        return rc, f[0], gv, H

    def circuit_projected_gradient(self, ufunc, udata, gates, wires, L):
        g = gates_arr(gates); w = np.ascontiguousarray(np.asarray(wires, np.int32).reshape(-1))
        f = np.zeros(1, cd); gv = np.zeros(8 * len(g))
        rc = self.lib.matchgate_circuit_unitary_target_and_projected_gradient(P(ufunc), P(udata), _p(g), len(g), _p(w), L, _p(f), _p(gv))
        return rc, f[0], gv

    def brickwall_target(self, ufunc, udata, vlist, perms, L):
        v = gates_arr(vlist); pp, rows = _perm_ptrs(perms, L); f = np.zeros(1, cd)
        rc = self.lib.matchgate_brickwall_unitary_target(P(ufunc), P(udata), _p(v), len(v), L, C.cast(pp, P), _p(f))
        return rc, f[0]

    def brickwall_target_and_gradient(self, ufunc, udata, vlist, perms, L):
        v = gates_arr(vlist); pp, rows = _perm_ptrs(perms, L); f = np.zeros(1, cd); dv = np.zeros((len(v), 8), cd)
        rc = self.lib.matchgate_brickwall_unitary_target_and_gradient(P(ufunc), P(udata), _p(v), len(v), L, C.cast(pp, P), _p(f), _p(dv))
        return rc, f[0], dv

    def brickwall_target_gradient_hessian(self, ufunc, udata, vlist, perms, L, ti=False, parallel=False):
        v = gates_arr(vlist); pp, rows = _perm_ptrs(perms, L); f = np.zeros(1, cd); dv = np.zeros((len(v), 8), cd)
        m = 8 * len(v); h = np.zeros((m, m), cd)
        if ti:
            fn = self.lib.matchgate_ti_brickwall_unitary_target_gradient_hessian
        elif parallel:
            fn = self.lib.parallel_matchgate_brickwall_unitary_target_gradient_hessian
        else:
            fn = self.lib.matchgate_brickwall_unitary_target_gradient_hessian
        rc = fn(P(ufunc), P(udata), _p(v), len(v), L, C.cast(pp, P), _p(f), _p(dv), _p(h))
        return rc, f[0], dv, h

    def brickwall_gradvec_hessmat(self, ufunc, udata, vlist, perms, L):
        v = gates_arr(vlist); pp, rows = _perm_ptrs(perms, L); f = np.zeros(1, cd)
        m = 8 * len(v); g = np.zeros(m); H = np.zeros((m, m))
        rc = self.lib.matchgate_brickwall_unitary_target_gradient_vector_hessian_matrix(P(ufunc), P(udata), _p(v), len(v), L, C.cast(pp, P),
                                                                                       _p(f), _p(g), _p(H))
        return rc, f[0], g, H

    def brickwall_projected_gradient(self, ufunc, udata, vlist, perms, L):
        v = gates_arr(vlist); pp, rows = _perm_ptrs(perms, L); f = np.zeros(1, cd); g = np.zeros(8 * len(v))
        rc = self.lib.matchgate_brickwall_unitary_target_and_projected_gradient(P(ufunc), P(udata), _p(v), len(v), L, C.cast(pp, P), _p(f), _p(g))
        return rc, f[0], g

    def brickwall_columns(self, ufunc, udata, vlist, perms, L, b0, b1, gradient=True):
        v = gates_arr(vlist); pp, rows = _perm_ptrs(perms, L); f = np.zeros(1, cd); dv = np.zeros((len(v), 8), cd)
        rc = self.lib.mg_brickwall_target_and_gradient_columns(P(ufunc), P(udata), _p(v), len(v), L, C.cast(pp, P), b0, b1, _p(f),
                                                               _p(dv) if gradient else None)
        return rc, f[0], dv

    # ------------------------------------------------------------------ device-resident plans
    def plan_brickwall(self, ufunc, udata, vlist, perms, L, what):
        v = gates_arr(vlist); pp, rows = _perm_ptrs(perms, L)
        h = self.lib.mg_plan_brickwall(P(ufunc), P(udata), _p(v), len(v), L, C.cast(pp, P), what)
        if not h:
            raise RuntimeError("mg_plan_brickwall failed: " + self.last_error())
        return h

    def plan_results(self, plan, nlayers, grad=False, hess=False, proj=False):
        f = np.zeros(1, cd)
        dv = np.zeros((nlayers, 8), cd) if grad else None
        m = 8 * nlayers
        h = np.zeros((m, m), cd) if hess else None
        g = np.zeros(m) if proj else None
        H = np.zeros((m, m)) if (proj and hess) else None
        rc = self.lib.mg_plan_results(P(plan), _p(f), _p(dv), _p(h), _p(g), _p(H))
        assert rc == 0, self.last_error()
        return f[0], dv, h, g, H

    # ------------------------------------------------------------------ algebra (matchgate.h)
    def _mg(self, name, *gs):
        gs = [gates_arr(g) for g in gs]
        out = np.zeros((1, 8), cd)
        getattr(self.lib, name)(*[_p(g) for g in gs], _p(out))
        return out[0]

    def multiply(self, a, b):
        return self._mg("multiply_matchgates", a, b)

    def project_tangent(self, u, z):
        return self._mg("project_tangent_matchgate", u, z)

    def polar(self, a):
        return self._mg("polar_matchgate_factor", a)

    def real_to_tangent(self, r, v):
        r = np.ascontiguousarray(r, np.float64); v = gates_arr(v); out = np.zeros((1, 8), cd)
        self.lib.real_to_tangent_matchgate(_p(r), _p(v), _p(out))
        return out[0]

    def tangent_to_real(self, v, z):
        v = gates_arr(v); z = gates_arr(z); r = np.zeros(8)
        self.lib.tangent_matchgate_to_real(_p(v), _p(z), _p(r))
        return r

    def project_gradient(self, vlist, dvlist):
        """Riemannian gradient vector [8 nlayers] of raw layer gradients: each conjugated and
        mapped by tangent_matchgate_to_real (reference src/matchgate_target.c:902-908)"""
        v = gates_arr(vlist)
        dv = gates_arr(dvlist)
        return np.concatenate([self.tangent_to_real(v[i], np.conj(dv[i])) for i in range(len(v))])

    def retract(self, u, eta):
        u = gates_arr(u); eta = np.ascontiguousarray(eta, np.float64); out = np.zeros((1, 8), cd)
        self.lib.retract_matchgate(_p(u), _p(eta), _p(out))
        return out[0]

    def truncated_cg(self, grad, hess, radius, maxiter, abstol=1e-8, reltol=1e-6):
        g = np.ascontiguousarray(grad, np.float64); h = np.ascontiguousarray(hess, np.float64); z = np.zeros_like(g)
        prm = TcgParams(maxiter, abstol, reltol)
        onb = self.lib.truncated_cg_hmat(_p(g), _p(h), len(g), radius, C.byref(prm), _p(z))
        return z, bool(onb)

    # ------------------------------------------------------------------ trust region
    def optimize_brickwall(self, ufunc, udata, vlist0, perms, L, niter, tcg_maxiter=None,
                           rho_trust=0.125, radius_init=0.01, maxradius=0.1):
        """riemannian_trust_region_optimize_hmat driven like the reference's
        optimize_matchgate_brickwall_circuit_hmat (src/mg_brickwall_opt.c:99-122):
        f and f_deriv_hess call this library's evaluations, retraction per layer."""
        v0 = gates_arr(vlist0); nl = len(v0); n = 8 * nl; m = 16 * nl
        pp, rows = _perm_ptrs(perms, L)
        lib = self.lib

        def f_cb(x, fdata, fc):
            fv = np.zeros(1, cd)
            rc = lib.matchgate_brickwall_unitary_target(P(ufunc), P(udata), C.cast(x, P), nl, L, C.cast(pp, P), _p(fv))
            if rc < 0:
                return -1.0
            fc[0] = fv[0].real; fc[1] = fv[0].imag
            return fv[0].real

        def fdh_cb(x, fdata, fc, grad, hess):
            fv = np.zeros(1, cd)
            rc = lib.matchgate_brickwall_unitary_target_gradient_vector_hessian_matrix(
                P(ufunc), P(udata), C.cast(x, P), nl, L, C.cast(pp, P), _p(fv), C.cast(grad, P), C.cast(hess, P))
            if rc < 0:
                return -1.0
            fc[0] = fv[0].real; fc[1] = fv[0].imag
            return fv[0].real

        def retract_cb(x, eta, rdata, xs):
            ax, ae, axs = (C.cast(q, C.c_void_p).value for q in (x, eta, xs))
            for i in range(nl):   # one gate = 16 doubles, one tangent vector = 8 doubles
                lib.retract_matchgate(P(ax + 128 * i), P(ae + 64 * i), P(axs + 128 * i))

        fcb, fdhcb, rcb = TargetFunc(f_cb), TargetGradHessFunc(fdh_cb), RetractFunc(retract_cb)
        prm = RtrParams()
        prm.tcg_params = TcgParams(tcg_maxiter if tcg_maxiter is not None else 2 * 16 * nl, 1e-8, 1e-6)
        prm.rho_trust, prm.radius_init, prm.maxradius = rho_trust, radius_init, maxradius
        f_iter = np.zeros(niter + 1); f_citer = np.zeros(niter + 1, cd); xf = np.zeros((nl, 8), cd)
        lib.riemannian_trust_region_optimize_hmat(fcb, fdhcb, None, rcb, None, n, _p(v0), m, C.byref(prm), niter,
                                                  _p(f_iter), _p(f_citer), _p(xf))
        return f_iter, f_citer, xf


_default = None


def default_lib():
    """The in-tree libmgcu.so (raises if it has not been built)."""
    global _default
    if _default is None:
        if not os.path.exists(DEFAULT_LIB):
            raise RuntimeError("libmgcu.so is missing: build it with rqcopt_hpc-matchgate_gb300/build.py "
                               "(this library has no CPU implementation to fall back to)")
        _default = MatchgateLib(DEFAULT_LIB)
    return _default
