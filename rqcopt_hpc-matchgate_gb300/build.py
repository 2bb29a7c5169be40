"""Build the GB300 matchgate library, in tree.

Compiles the CUDA layer (csrc/cuda/*.cu, sm_103a only) with nvcc and the C host
layer (csrc/host/*.c, the reference-compatible API) with gcc, in parallel, and links
``_build/libmgcu.so``.  Re-running only rebuilds what changed.

    python rqcopt_hpc-matchgate_gb300/build.py [-f]
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libmgcu.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INC = ["-I", os.path.join(ROOT, "include"), "-I", os.path.join(HERE, "csrc")]


def _sources():
    cu = sorted(glob.glob(os.path.join(HERE, "csrc", "cuda", "*.cu")))
    c = sorted(glob.glob(os.path.join(HERE, "csrc", "host", "*.c")))
    hdr = (glob.glob(os.path.join(HERE, "csrc", "*.h")) + glob.glob(os.path.join(HERE, "csrc", "cuda", "*.cuh"))
           + glob.glob(os.path.join(HERE, "csrc", "host", "*.h"))
           + glob.glob(os.path.join(ROOT, "include", "*.h")))
    return cu, c, hdr


def _obj(src):
    return os.path.join(OUT, os.path.basename(src) + ".o")


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    cu, c, hdr = _sources()
    jobs = []
    for s in cu:
        o = _obj(s)
        if force or _stale(o, [s, __file__] + hdr):
            # the engine is one large translation unit: let nvcc optimise its kernels in parallel
            split = ["--split-compile=0"] if os.path.basename(s) == "mgcu_engine.cu" else []
            jobs.append(([NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"] + split + INC
                         + ["-c", s, "-o", o], s))
    for s in c:
        o = _obj(s)
        if force or _stale(o, [s, __file__] + hdr):
            jobs.append((["gcc", "-O2", "-std=gnu11", "-fPIC", "-Wall", "-Wno-unused-function"] + INC
                         + ["-c", s, "-o", o], s))
    procs = [(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True), cmd, s) for cmd, s in jobs]
    failed = []
    for p, cmd, s in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((s, " ".join(cmd), out))
        elif verbose and out.strip():
            print(out)
    if failed:
        for s, cmd, out in failed:
            sys.stderr.write(f"--- {s}\n{cmd}\n{out}\n")
        raise RuntimeError("building libmgcu.so failed")
    objs = [_obj(s) for s in cu + c]
    if force or jobs or _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread", "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("linking libmgcu.so failed")
    return LIB


if __name__ == "__main__":
    print(build(force="-f" in sys.argv, verbose="-v" in sys.argv))
