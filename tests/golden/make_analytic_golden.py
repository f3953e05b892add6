"""Regenerate ``analytic_fields.npz`` beside this script: the fields of the
reference's own analytic Stokes solutions at seeded points, for every case of
``analytic_cases.py``.

The values come from the reference's C and C++ solution code, compiled from the
reference tree by ``oracle/ref_analytic.py`` (set UW_REFERENCE_TREE to the tree
when it is not at the default location):

    python tests/golden/make_analytic_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from oracle import ref_analytic  # noqa: E402
from analytic_cases import CASES, FIELDS  # noqa: E402


def main():
    rng = np.random.default_rng(20261204)
    out = {}
    for i, (name, prm, _, dim) in enumerate(CASES):
        x = rng.uniform(0.01, 0.99, (24 if dim == 2 else 12, dim))
        ref = ref_analytic.evaluate(name, prm, x)
        out["%d/points" % i] = x
        for f in FIELDS:
            out["%d/%s" % (i, f)] = ref[f]
    np.savez_compressed(os.path.join(HERE, "analytic_fields.npz"), **out)


if __name__ == "__main__":
    main()
