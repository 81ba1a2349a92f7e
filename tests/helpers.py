"""Shared helpers of the test suite (inputs, tolerances, comparisons)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_vectors.npz")


def golden():
    return np.load(GOLDEN)


def rel_err(a, b):
    """max |a - b| / max |b| (the normwise check used throughout)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / den)


def fro_rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


# tolerances: FP64 path vs the FP64 oracle (the stated 1e-12 relative);
# FP32 path (FP32 arithmetic) vs the FP64 oracle
TOL_F64 = 1e-12
TOL_F32 = 2e-5
