"""Records golden colourings of FunctionsPacking from the reference MGmol's
own src/tools/coloring.cc (compiled unmodified against the single-task mpi
shim by oracle/build_ref.sh -> oracle/_ref/libmgref.so).

The overlap pattern of each case comes from the oracle's restatement of
the one-task subdomain geometry (oracle.pack_overlap); the reference then
colours it greedily and by RLF.  Inputs and colours go to
tests/golden/pack_vectors.npz; tests/test_pack_cpu.py checks the library's
mgx_pack_functions and the oracle's colourings against them.  Re-run after
changing the generator:

    oracle/build_ref.sh && python tests/golden/make_pack_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402

# (grid, lengths, orbitals, radius range, sub-boxes, ghosts, seed)
CASES = [((64, 64, 64), (22.4, 22.4, 22.4), 64, (2.0, 4.0), 8, 1, 11),
         ((96, 48, 48), (28.8, 14.4, 14.4), 90, (1.0, 3.0), 12, 1, 12),
         ((40, 32, 48), (12.0, 9.6, 14.4), 50, (0.3, 1.0), 8, 2, 13),
         ((64, 64, 64), (22.4, 22.4, 22.4), 33, (2.0, 4.0), 1, 1, 14)]


def main():
    if O.ref_lib() is None:
        raise SystemExit("oracle/_ref/libmgref.so missing: run oracle/build_ref.sh first")
    out = {}
    for k, (n, ll, nf, (rlo, rhi), sd, ghosts, seed) in enumerate(CASES):
        rng = np.random.default_rng(seed)
        centers = rng.uniform(0.0, 1.0, size=(nf, 3)) * np.asarray(ll)[None, :]
        radii = rng.uniform(rlo, rhi, size=nf).astype(np.float32)
        ov = O.pack_overlap(n, ll, centers, radii, sd, ghosts)
        out[f"c{k}_grid"] = np.asarray(n, dtype=np.int32)
        out[f"c{k}_ll"] = np.asarray(ll)
        out[f"c{k}_centers"] = centers
        out[f"c{k}_radii"] = radii
        out[f"c{k}_subdiv"] = np.asarray([sd, ghosts], dtype=np.int32)
        out[f"c{k}_overlap"] = ov
        for rlf in (0, 1):
            col, nc = O.ref_pack_colors(ov, rlf)
            out[f"c{k}_colors{rlf}"] = col
            out[f"c{k}_ncolors{rlf}"] = np.asarray([nc], dtype=np.int32)
    out["ncases"] = np.asarray([len(CASES)], dtype=np.int32)
    np.savez_compressed(os.path.join(HERE, "pack_vectors.npz"), **out)


if __name__ == "__main__":
    main()
