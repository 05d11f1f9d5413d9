"""Copy the reference's SFB test fixtures into tests/golden/.

The reference keeps one end-to-end fixture for the decomposition path
(test/test_data/, used by test/python/decomposition_test.py:8-73):
  gaussian_catalog.txt           445 Cartesian points (x y z), rmax 2500
  gaussian_catalog.python.k_ln   10x10 k_ln
  gaussian_catalog.python.c_ln   10x10 C_ln of the raw method
  gaussian_catalog.pythonrev.*   the same for the pixelized method at nside 64
The files are copied byte for byte; the GPU test machines have no reference tree.
Run from the repository root:
    python tests/golden/make_golden.py REFERENCE_ROOT
(or with the reference tree in $CATANA_REFERENCE_DIR).
"""
import os
import shutil
import sys

NAMES = ["gaussian_catalog.txt",
         "gaussian_catalog.python.k_ln", "gaussian_catalog.python.c_ln",
         "gaussian_catalog.pythonrev.k_ln", "gaussian_catalog.pythonrev.c_ln"]


def main(ref_root=None):
    ref_root = ref_root or os.environ.get("CATANA_REFERENCE_DIR")
    if not ref_root:
        sys.exit("usage: make_golden.py REFERENCE_ROOT (or set CATANA_REFERENCE_DIR)")
    src = os.path.join(ref_root, "test", "test_data")
    dst = os.path.dirname(os.path.abspath(__file__))
    for n in NAMES:
        shutil.copyfile(os.path.join(src, n), os.path.join(dst, n))
        print("copied", n)


if __name__ == "__main__":
    main(*sys.argv[1:])
