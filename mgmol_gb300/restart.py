"""Snapshots of a run's arrays through the C ABI (mgx_snapshot_*).

MGmol writes restart files with parallel HDF5 (MGmol::dumpRestart,
src/MGmol.cc:1101-1127; HDFrestart, src/HDFrestart.cc) and reads orbitals
back function by function (LocGridOrbitals::read_func_hdf5,
src/LocGridOrbitals.cc:1182).  HDF5 is not available to this build, so a
snapshot is one flat file: a JSON header (grid, caller metadata, each
array's type, shape, offset and CRC-32) and the raw arrays, 4096-byte
aligned.  Device tensors stream to and from the file through pinned host
buffers inside the library.

    save(path, grid=(n, ll), meta={"sweep": 30}, psi=psi, V=V, unet=params)
    header(path)                      # the parsed JSON header
    load(path, "psi", out=psi)        # into an existing tensor (device or host)
    load(path, "V")                   # a new host tensor
"""
import ctypes
import json

import numpy as np
import torch

from . import capi

_TYPES = {torch.float64: capi.SNAP_F64, torch.float32: capi.SNAP_F32,
          torch.int32: capi.SNAP_I32, torch.uint8: capi.SNAP_U8}
_TORCH = {"f64": torch.float64, "f32": torch.float32, "i32": torch.int32, "u8": torch.uint8}


def _tensor(a):
    t = torch.from_numpy(np.ascontiguousarray(a)) if isinstance(a, np.ndarray) else a
    if not t.is_contiguous():
        t = t.contiguous()
    if t.dtype not in _TYPES:
        raise TypeError(f"snapshot arrays are float64, float32, int32 or uint8, not {t.dtype}")
    if t.dim() > 4:
        raise ValueError("snapshot arrays have at most 4 dimensions")
    return t


def save(path, grid=None, meta=None, stream=None, **arrays):
    """Writes the named arrays (torch tensors on any device, or numpy) and
    the grid ((n, ll) or None) with `meta` (anything json.dumps takes)."""
    keep = {k: _tensor(v) for k, v in arrays.items()}
    ds = (capi.Dataset * max(1, len(keep)))()
    for i, (name, t) in enumerate(keep.items()):
        ds[i].name = name.encode()
        ds[i].type = _TYPES[t.dtype]
        ds[i].ndim = t.dim()
        for k in range(t.dim()):
            ds[i].shape[k] = t.shape[k]
        ds[i].data = t.data_ptr() if t.numel() else None
    g = None
    if grid is not None:
        g = ctypes.byref(capi.Grid.make(grid[0], grid[1]))
    m = json.dumps(meta).encode() if meta is not None else None
    if any(t.is_cuda for t in keep.values()):
        torch.cuda.current_stream().synchronize()
    capi._check(capi.load().mgx_snapshot_write(str(path).encode(), g, m, len(keep), ds,
                                               capi._stream(stream) if any(
                                                   t.is_cuda for t in keep.values()) else None))


def header(path):
    """The snapshot's JSON header as a dict."""
    L = capi.load()
    n = ctypes.c_size_t(0)
    capi._check(L.mgx_snapshot_header(str(path).encode(), None, 0, ctypes.byref(n)))
    buf = ctypes.create_string_buffer(n.value + 1)
    capi._check(L.mgx_snapshot_header(str(path).encode(), buf, n.value + 1, None))
    return json.loads(buf.value.decode())


def load(path, name, out=None, device="cpu", stream=None):
    """Array `name` into `out` (a contiguous tensor of its size, device or
    host), or into a new tensor on `device`; the CRC-32 is checked."""
    if out is None:
        d = next((x for x in header(path)["datasets"] if x["name"] == name), None)
        if d is None:
            raise capi.MgxError(capi.MGX_BAD_ARG, f"snapshot has no dataset '{name}'")
        out = torch.empty(d["shape"], dtype=_TORCH[d["type"]], device=device)
    if not out.is_contiguous():
        raise ValueError("out must be contiguous")
    nb = out.numel() * out.element_size()
    capi._check(capi.load().mgx_snapshot_read(str(path).encode(), name.encode(),
                                              out.data_ptr() if nb else None, nb,
                                              capi._stream(stream) if out.is_cuda else None))
    return out
