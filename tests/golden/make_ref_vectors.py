"""Golden vectors from the reference's own code: builds the reference's
functions for the CPU (oracle/ref/ref_build.py, from the reference source
tree), runs them on the pin inputs (oracle/ref/pins.py) and writes what they
compute to tests/golden/ref_vectors.npz. tests/test_oracle_reference_pins.py
checks the oracle against that file.

  python tests/golden/make_ref_vectors.py [REF_DIR]
"""
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import pins  # noqa: E402
import ref_build  # noqa: E402


def main():
    ref_dir = sys.argv[1] if len(sys.argv) > 1 else ref_build.REF_DIR
    if not ref_build.build(ref_dir):
        sys.exit("the reference source is not at %s" % ref_dir)
    L = pins.reference_lib(build=False)
    with tempfile.TemporaryDirectory() as d:
        scene = pins.write_scene(d)
        R = pins.reference_outputs(L, scene, os.path.join(ROOT, "data"), pins.inputs())
    path = os.path.join(HERE, "ref_vectors.npz")
    np.savez_compressed(path, **pins.pack(R))
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
