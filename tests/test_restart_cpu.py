"""Snapshots (mgx_snapshot_*, mgmol_gb300.restart) of host arrays: the
round trip of every element type, the header, the CRC-32 of a known input,
and the refusals (missing array, size mismatch, corrupted data, bad name)."""
import zlib

import numpy as np
import pytest
import torch

from mgmol_gb300 import capi, restart


def test_round_trip_and_header(tmp_path):
    rng = np.random.default_rng(5)
    psi = rng.standard_normal((3, 8 * 8 * 8)).astype(np.float32)
    V = rng.standard_normal(8 * 8 * 8)
    idx = np.arange(7, dtype=np.int32)
    raw = np.frombuffer(b"mgx", dtype=np.uint8).copy()
    p = tmp_path / "snap.bin"
    restart.save(p, grid=((8, 8, 8), (2.8, 2.8, 2.8)), meta={"sweep": 12, "gemm": "bf16x3"},
                 psi=psi, V=V, idx=idx, raw=raw)
    h = restart.header(p)
    assert h["format"] == "mgx-snapshot" and h["grid"]["n"] == [8, 8, 8]
    assert h["meta"] == {"sweep": 12, "gemm": "bf16x3"}
    names = [d["name"] for d in h["datasets"]]
    assert names == ["psi", "V", "idx", "raw"]
    for d in h["datasets"]:
        assert d["offset"] % 4096 == 0
    # the CRC-32 in the header is the standard one of the bytes
    d = h["datasets"][0]
    assert int(d["crc32"], 16) == zlib.crc32(psi.tobytes())
    assert np.array_equal(restart.load(p, "psi").numpy(), psi)
    assert np.array_equal(restart.load(p, "V").numpy(), V)
    assert np.array_equal(restart.load(p, "idx").numpy(), idx)
    assert restart.load(p, "raw").numpy().tobytes() == b"mgx"
    out = torch.empty(3, 8 * 8 * 8, dtype=torch.float32)
    restart.load(p, "psi", out=out)
    assert np.array_equal(out.numpy(), psi)


def test_last_array_filling_its_aligned_block(tmp_path):
    # an array whose size is a multiple of the 4096-byte alignment, last in
    # the file: its final byte is data, not padding
    a = np.arange(1024, dtype=np.float32) + 1.0      # 4096 bytes
    b = np.arange(512, dtype=np.float64) - 3.5       # 4096 bytes
    p = tmp_path / "aligned.bin"
    restart.save(p, a=a, b=b)
    assert np.array_equal(restart.load(p, "a").numpy(), a)
    assert np.array_equal(restart.load(p, "b").numpy(), b)


def test_refusals(tmp_path):
    p = tmp_path / "snap.bin"
    a = np.arange(1000, dtype=np.float64)
    restart.save(p, a=a)
    with pytest.raises(capi.MgxError):
        restart.load(p, "b")
    with pytest.raises(capi.MgxError):
        restart.load(p, "a", out=torch.empty(999, dtype=torch.float64))
    # one flipped byte in the data fails the checksum
    off = restart.header(p)["datasets"][0]["offset"]
    b = bytearray(p.read_bytes())
    b[off + 17] ^= 0x40
    p.write_bytes(bytes(b))
    with pytest.raises(capi.MgxError) as e:
        restart.load(p, "a")
    assert "checksum" in str(e.value)
    with pytest.raises(capi.MgxError):
        restart.save(tmp_path / "x.bin", **{'bad"name': a})
    (tmp_path / "junk.bin").write_bytes(b"not a snapshot at all" * 10)
    with pytest.raises(capi.MgxError):
        restart.header(tmp_path / "junk.bin")
