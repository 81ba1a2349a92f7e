"""Records the position tables of pb::Grid::getSinCosFunctions (the
factors of SpreadsAndCenters' centres) from the reference MGmol's own
src/pb/Grid.cc, compiled unmodified against the single-task shims by
oracle/build_ref.sh -> oracle/_ref/libmgref.so, into
tests/golden/centers_vectors.npz; tests/test_centers_cpu.py checks the
oracle's restatement against them.  Re-run after changing the generator:

    oracle/build_ref.sh && python tests/golden/make_centers_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402

GRIDS = [((64, 48, 40), (22.4, 16.8, 14.0)), ((37, 29, 31), (10.1, 9.3, 8.7)),
         ((192, 192, 192), (48.0, 48.0, 48.0))]


def main():
    if O.ref_lib() is None:
        raise SystemExit("oracle/_ref/libmgref.so missing: run oracle/build_ref.sh first")
    out = {}
    for k, (n, ll) in enumerate(GRIDS):
        out[f"g{k}_n"] = np.asarray(n, dtype=np.int32)
        out[f"g{k}_ll"] = np.asarray(ll)
        out[f"g{k}_tables"] = O.sincos_tables(n, ll, ref=True)
    out["ngrids"] = np.asarray([len(GRIDS)], dtype=np.int32)
    np.savez_compressed(os.path.join(HERE, "centers_vectors.npz"), **out)


if __name__ == "__main__":
    main()
