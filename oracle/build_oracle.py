"""Build recipe for the oracle (test infrastructure only).

Two things are built here, both into git-ignored folders:

* ``oracle/_build/libmgoracle.so`` -- this project's own C restatement of the
  reference algorithm (``oracle/mg_oracle.c``), compiled with OpenMP.  It builds on
  any machine with gcc (x86 or Arm) and is the checker used by the GPU parity tests
  and the timed CPU baseline.
* ``oracle/_ref/libref_mg*.so`` -- the reference library itself, compiled directly
  from its own source files where they lie (``src/*.c`` of the reference checkout),
  with the two stand-in headers in ``oracle/shim/``.  Only possible where the
  reference checkout exists; used by the CPU tests to pin the restatement.

Nothing here is imported by the product library.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = os.environ.get("MG_REFERENCE_SRC", "/root/reference/src")

REF_FILES = ["gate.c", "matchgate.c", "matchgate_brickwall.c", "matchgate_target.c",
             "mg_brickwall_opt.c", "quantum_circuit.c", "statevector.c", "trust_region.c", "util.c"]

# name -> extra defines; all variants use the complex128 build of the reference
REF_VARIANTS = {
    "libref_mg.so": [],
    "libref_mg_omp.so": ["-DSTATEVECTOR_PARALLELIZATION"],
    "libref_mg_ti.so": ["-DTRANSLATIONAL_INVARIANCE"],
}


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("oracle build step failed: " + cmd[-1])


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_oracle(force=False):
    """Compile the C restatement into oracle/_build/libmgoracle.so."""
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    src = os.path.join(HERE, "mg_oracle.c")
    hdr = os.path.join(HERE, "mg_oracle.h")
    out = os.path.join(out_dir, "libmgoracle.so")
    if force or _stale(out, [src, hdr, __file__]):
        _run(["gcc", "-O3", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-Wall", "-o", out, src, "-lm"])
    return out


def build_reference(force=False):
    """Compile the reference library from its own sources (only where they exist)."""
    if not os.path.isdir(REF_SRC):
        return []
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    srcs = [os.path.join(REF_SRC, f) for f in REF_FILES]
    shims = [os.path.join(HERE, "shim", "hdf5.h"), os.path.join(HERE, "shim", "cblas.h")]
    outs = []
    for name, defs in REF_VARIANTS.items():
        out = os.path.join(out_dir, name)
        if force or _stale(out, srcs + shims + [__file__]):
            cmd = ["gcc", "-O3", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-w",
                   "-DCOMPLEX_CIRCUIT"] + defs + [
                   "-I", os.path.join(HERE, "shim"), "-I", REF_SRC, "-o", out] + srcs + ["-lm"]
            _run(cmd)
        outs.append(out)
    return outs


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_reference(force="-f" in sys.argv))
