"""Regenerate the reference's golden test vectors as small .npz fixtures.

The reference keeps its known-answer data in HDF5 files written by seeded Python
generators (``test/test_gate.py``, ``test/test_matchgate.py``,
``test/test_matchgate_brickwall.py``, ``test/test_matchgate_target.py``).  h5py is
not installed here, so this script runs those generators unchanged against an
in-memory stand-in for ``h5py.File`` (a dict), and saves every dataset it wrote to
``tests/golden/<fixture>.npz``.  Nothing is written into the reference checkout.

Each regenerated dataset is then searched for, byte for byte, in the HDF5 file the
reference ships (``test/data/<fixture>.hdf5``); the outcome per dataset is recorded
in ``tests/golden/MANIFEST.txt`` so the fixtures are pinned to the shipped files.

Run (needs the reference checkout; the committed .npz files are what tests use):
    python tests/golden/gen_golden.py [/path/to/reference]
"""
import io
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MG_REFERENCE", "")
if not REF:
    sys.exit("usage: gen_golden.py <reference checkout> (or set MG_REFERENCE)")
REF_TEST = os.path.join(REF, "test")

CAPTURED = {}


class _Group(dict):
    """A minimal stand-in for an h5py File: path-keyed datasets plus attrs."""

    def __init__(self, path):
        super().__init__()
        self.path = path
        self.attrs = {}

    def __setitem__(self, key, value):
        super().__setitem__(key, np.asarray(value))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False

    def close(self):
        CAPTURED[os.path.basename(self.path)] = self


def _install_fake_h5py():
    mod = types.ModuleType("h5py")
    mod.File = lambda path, mode="r": _Group(path)
    sys.modules["h5py"] = mod


# (generator module, functions) -- the fixtures the reference's C tests read
GENERATORS = [
    ("test_gate", ["apply_matchgate_data", "apply_matchgate_backward_data",
                   "apply_matchgate_backward_array_data", "apply_matchgate_to_array_data",
                   "apply_matchgate_placeholder_data"]),
    ("test_matchgate", ["real_to_tangent_matchgate_data", "multiply_data_matchgate",
                        "project_tangent_matchgate_data", "polar_matchgate_factor_data"]),
    ("test_matchgate_brickwall", ["apply_matchgate_brickwall_unitary_data",
                                  "matchgate_brickwall_unitary_backward_data",
                                  "matchgate_brickwall_unitary_backward_hessian_data"]),
    ("test_matchgate_target", ["matchgate_circuit_unitary_target_data",
                               "matchgate_brickwall_unitary_target_data",
                               "matchgate_brickwall_unitary_target_gradient_hessian_data",
                               "matchgate_brickwall_unitary_target_gradient_vector_hessian_matrix_data",
                               "matchgate_ti_brickwall_unitary_target_gradient_hessian_data",
                               "matchgate_ti_brickwall_unitary_target_gradient_hessian_data2",
                               "matchgate_ti_brickwall_unitary_target_gradient_hessian_data3"]),
]


def main():
    sys.dont_write_bytecode = True
    _install_fake_h5py()
    sys.path.insert(0, REF_TEST)
    manifest = []
    for modname, funcs in GENERATORS:
        mod = __import__(modname)
        for fn in funcs:
            CAPTURED.clear()
            stdout = sys.stdout
            sys.stdout = io.StringIO()
            try:
                getattr(mod, fn)()
            finally:
                sys.stdout = stdout
            for fname, grp in CAPTURED.items():
                stem = os.path.splitext(fname)[0]
                arrays = {k.replace("/", "__"): v for k, v in grp.items()}
                np.savez_compressed(os.path.join(HERE, stem + ".npz"), **arrays)
                shipped = os.path.join(REF_TEST, "data", fname)
                blob = open(shipped, "rb").read() if os.path.exists(shipped) else None
                n_found = 0
                for k, v in grp.items():
                    raw = np.ascontiguousarray(v).tobytes()
                    found = blob is not None and raw in blob
                    n_found += found
                    if not found:
                        manifest.append(f"  {k:24s} shape={tuple(v.shape)!s:16s} NOT found by byte search")
                manifest.append(f"{stem}: {n_found}/{len(grp)} datasets byte-identical to the shipped HDF5 file")
                print(manifest[-1])
    with open(os.path.join(HERE, "MANIFEST.txt"), "w") as f:
        f.write("Regenerated by tests/golden/gen_golden.py from the reference's own seeded generators.\n")
        f.write("Dataset names use '__' where the HDF5 path used '/'.\n\n")
        f.write("\n".join(manifest) + "\n")


if __name__ == "__main__":
    main()
