"""CPU-only checks of the C ABI: the library loads without a GPU, exports every function
declared in include/*.h, keeps the reference's struct layouts, runs its host-side helpers
correctly, refuses GPU work loudly when no GPU is present, and links the reference's own
optimiser source unchanged."""
import ctypes as C
import glob
import os
import re
import subprocess

import numpy as np
import pytest

import mgcu
from conftest import REF_SRC, ROOT, random_gates, udist

INCLUDE = os.path.join(ROOT, "include")


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(INCLUDE, "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"static inline[^{]*\{.*?\n\}", "", src, flags=re.S)
        src = re.sub(r"typedef[^;]*;", "", src)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(([^;{}]*)\)\s*;", src, flags=re.S):
            names.add(m.group(1))
    return sorted(names)


def test_exports_every_declared_function(mglib):
    names = declared_functions()
    assert len(names) > 70
    missing = [n for n in names if not hasattr(mglib.lib, n)]
    assert not missing, missing


def test_struct_layouts():
    # struct matchgate is 8 complex128; statevector is {pointer, int}
    assert C.sizeof(mgcu.StateVector) == 16
    assert C.sizeof(mgcu.StateVectorArray) == 16
    assert C.sizeof(mgcu.CircuitCache) == 16
    assert C.sizeof(mgcu.RtrParams) == 72


def test_host_helpers_match_oracle(mglib, oracle):
    rng = np.random.default_rng(0)
    for _ in range(5):
        a, b = random_gates(2, rng, scale=1.0)
        assert udist(mglib.multiply(a, b), oracle.mg_multiply(a, b)) < 1e-15
        assert udist(mglib.polar(a), oracle.mg_polar(a)) < 1e-14
        u = random_gates(1, rng, unitary=True)[0]
        assert udist(mglib.project_tangent(u, a), oracle.mg_project_tangent(u, a)) < 1e-15
        r = rng.standard_normal(8)
        assert udist(mglib.real_to_tangent(r, u), oracle.mg_real_to_tangent(r, u)) < 1e-15
        assert udist(mglib.tangent_to_real(u, a), oracle.mg_tangent_to_real(u, a)) < 1e-15
    # statevector allocation and transposition (src/statevector.c:49-72)
    sv = mgcu.StateVector()
    assert mglib.lib.allocate_statevector(5, C.byref(sv)) == 0 and sv.nqubits == 5
    assert sv.data % 64 == 0
    psi = np.ctypeslib.as_array(C.cast(sv.data, C.POINTER(C.c_double)), shape=(64,)).view(np.complex128)
    psi[:] = np.arange(32) + 1j
    out = mgcu.StateVector()
    mglib.lib.allocate_statevector(5, C.byref(out))
    perm = np.array([2, 0, 1, 4, 3], np.int32)
    mglib.lib.transpose_statevector(C.byref(sv), C.c_void_p(perm.ctypes.data), C.byref(out))
    res = np.ctypeslib.as_array(C.cast(out.data, C.POINTER(C.c_double)), shape=(64,)).view(np.complex128).copy()
    expect = psi.reshape([2] * 5).transpose(perm).reshape(-1)
    assert np.array_equal(res, expect)
    mglib.lib.free_statevector(C.byref(sv)); mglib.lib.free_statevector(C.byref(out))
    assert sv.data is None or sv.data == 0


def test_gpu_work_fails_loudly_without_gpu(mglib):
    if os.path.exists("/dev/nvidiactl"):
        pytest.skip("a GPU is present")
    rng = np.random.default_rng(1)
    rc, f = mglib.brickwall_target(0, None, random_gates(2, rng), np.array([np.arange(6)] * 2, np.int32), 6)
    assert rc == -5
    assert "CUDA" in mglib.last_error() or "device" in mglib.last_error()


def test_reference_optimiser_links(mglib, tmp_path):
    """the reference's src/mg_brickwall_opt.c compiles against include/ and links to
    libmgcu.so with every symbol resolved"""
    src = os.path.join(REF_SRC, "mg_brickwall_opt.c")
    if not os.path.exists(src):
        pytest.skip("reference sources not present on this machine")
    # compile a temporary copy, so its quoted includes resolve to include/ rather than
    # to the reference's own headers beside it
    import shutil
    for f in ("mg_brickwall_opt.c", "mg_brickwall_opt.h"):
        shutil.copy(os.path.join(REF_SRC, f), tmp_path / f)
    obj = tmp_path / "opt.o"
    subprocess.run(["gcc", "-O2", "-std=gnu11", "-fPIC", "-DCOMPLEX_CIRCUIT", "-I", INCLUDE, "-c", str(tmp_path / "mg_brickwall_opt.c"),
                    "-o", str(obj)], check=True)
    main = tmp_path / "main.c"
    main.write_text("#include \"mg_brickwall_opt.h\"\nint main(void){ return (int)(long)&optimize_matchgate_brickwall_circuit_hmat == 0; }\n")
    exe = tmp_path / "linkcheck"
    libdir = os.path.dirname(mglib.path)
    r = subprocess.run(["gcc", "-std=gnu11", "-DCOMPLEX_CIRCUIT", "-I", INCLUDE, "-I", str(tmp_path), str(main), str(obj), "-L", libdir, "-lmgcu",
                        "-Wl,-rpath," + libdir, "-Wl,--no-undefined", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_c_driver_builds_against_the_headers(trdriver):
    """tests/helpers/mg_test_tr_driver.c (a C caller with the reference's optimiser glue)
    compiles against include/ and links to libmgcu.so with every symbol resolved"""
    assert hasattr(trdriver, "mgt_optimize_brickwall_hmat")
