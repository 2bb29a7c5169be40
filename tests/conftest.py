"""Shared fixtures.

* ``oracle``   -- the C restatement of the reference (oracle/), the checker;
* ``reflib``   -- the reference library compiled from its own sources (only where the
                  reference checkout exists; tests using it are skipped elsewhere);
* ``helpers``  -- test-side target maps (tests/helpers/mg_test_ufuncs.c);
* ``mglib``    -- the library under test, bound through its C API;
* ``golden``   -- the regenerated reference fixtures in tests/golden/.
Tests that need a GPU carry ``@pytest.mark.gpu``.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "rqcopt_hpc-matchgate_gb300")
for p in (os.path.join(ROOT, "oracle"), PKG, os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)

# where the reference sources lie: the oracle recipe owns that default (MG_REFERENCE_SRC overrides);
# tests that need them skip when they are absent (as on a machine without the reference)
from build_oracle import REF_SRC  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def oracle():
    import build_oracle as obuild
    obuild.build_oracle()
    import oracle as orc
    return orc


@pytest.fixture(scope="session")
def reflib():
    if not os.path.isdir(REF_SRC):
        pytest.skip("reference sources not present on this machine")
    import build_oracle as obuild
    outs = obuild.build_reference()
    import mgcu
    return mgcu.MatchgateLib(outs[0])


@pytest.fixture(scope="session")
def reflib_ti():
    if not os.path.isdir(REF_SRC):
        pytest.skip("reference sources not present on this machine")
    import build_oracle as obuild
    outs = obuild.build_reference()
    import mgcu
    return mgcu.MatchgateLib(outs[2])


@pytest.fixture(scope="session")
def helpers():
    out_dir = os.path.join(ROOT, "tests", "_build")
    os.makedirs(out_dir, exist_ok=True)
    src = os.path.join(ROOT, "tests", "helpers", "mg_test_ufuncs.c")
    so = os.path.join(out_dir, "libmgtest.so")
    if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-o", so, src], check=True)
    return ctypes.CDLL(so)


@pytest.fixture(scope="session")
def trdriver(mglib):
    """tests/helpers/mg_test_tr_driver.c built against include/ and linked to libmgcu.so
    (fails, not skips, when it cannot be built)"""
    out_dir = os.path.join(ROOT, "tests", "_build")
    os.makedirs(out_dir, exist_ok=True)
    src = os.path.join(ROOT, "tests", "helpers", "mg_test_tr_driver.c")
    so = os.path.join(out_dir, "libmgtrdriver.so")
    libdir = os.path.dirname(mglib.path)
    subprocess.run(["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-DCOMPLEX_CIRCUIT", "-I", os.path.join(ROOT, "include"),
                    "-o", so, src, "-L", libdir, "-lmgcu", "-Wl,-rpath," + libdir, "-Wl,--no-undefined"], check=True)
    return ctypes.CDLL(so)


@pytest.fixture(scope="session")
def mglib():
    import importlib.util
    spec = importlib.util.spec_from_file_location("mg_pkg_build", os.path.join(PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    path = mod.build()
    import mgcu
    return mgcu.MatchgateLib(path)


def cplx(a):
    """(..., 2) float64 interleaved -> complex128"""
    a = np.asarray(a)
    if a.dtype.kind == "c":
        return a
    return a[..., 0] + 1j * a[..., 1]


class Golden:
    def __init__(self, name):
        self.d = np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))

    def __getitem__(self, k):
        return self.d[k.replace("/", "__")]

    def c(self, k):
        return cplx(self[k])

    def gate(self, center, corner):
        return np.concatenate([self.c(center).reshape(4), self.c(corner).reshape(4)])


@pytest.fixture(scope="session")
def golden():
    return Golden


def udist(a, b):
    """uniform (max-abs) distance, as the reference's tests use (src/util.c:24-33)"""
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)))) if np.size(a) else 0.0


def rel(a, b):
    """relative 2-norm error of a against the reference value b"""
    a = np.asarray(a); b = np.asarray(b)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def crandn(shape, rng):
    return (rng.normal(size=shape) + 1j * rng.normal(size=shape)) / np.sqrt(2)


def random_gates(n, rng, unitary=False, scale=0.5):
    """n matchgates (n, 8): Gaussian 2x2 blocks, or Haar U(2) blocks via QR with phase fix"""
    out = np.zeros((n, 8), np.complex128)
    for i in range(n):
        for blk in range(2):
            a = crandn((2, 2), rng)
            if unitary:
                q, r = np.linalg.qr(a)
                q = q * (np.diag(r) / np.abs(np.diag(r)))
                a = q
            else:
                a = scale * a
            out[i, 4 * blk:4 * blk + 4] = a.reshape(4)
    return out


def brickwall_perms(L, nlayers, rng=None):
    """random permutations (reference tests) or alternating nearest-neighbour layers"""
    if rng is not None:
        return np.array([rng.permutation(L) for _ in range(nlayers)], dtype=np.int32)
    even = np.arange(L)
    odd = np.roll(np.arange(L), -1)
    return np.array([even if i % 2 == 0 else odd for i in range(nlayers)], dtype=np.int32)


def hash_target(L):
    """the reference tests' index-hash linear map (test/test_matchgate_target.c:20-34) as a matrix"""
    n = 1 << L
    U = np.zeros((n, n), np.complex128)
    for i in range(n):
        U[i, ((i + 3) * 113) % n] += -1.1 + 0.8j
        U[i, ((i + 9) * 173) % n] += 0.4 - 0.7j
        U[i, i] += 0.5 + 0.1j
        U[i, ((i + 4) * 199) % n] += -0.3 + 0.2j
    return U
