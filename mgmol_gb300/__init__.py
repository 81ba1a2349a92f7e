"""mgmol_gb300: MGmol's per-iteration orbital hot path on one GB300 (sm_103a).

The compute lives in the C-ABI library libmgx.so (include/mgx.h), built from
mgmol_gb300/csrc by mgmol_gb300/build.py.  `capi` binds it for torch device
tensors; `synth` makes the seeded synthetic workloads; `sweep` composes one
orbital sweep (H psi, Gram / H matrices, FP64 Cholesky / inverse / trace,
V-cycle preconditioner).  C++ callers include mgmol_gb300/cpp/mgmol_adaptor.h,
which offers MGmol's own operator classes on top of the same C ABI.
"""
from . import capi, synth  # noqa: F401

__all__ = ["capi", "synth"]
