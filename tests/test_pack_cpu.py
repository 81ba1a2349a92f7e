"""Function packing (mgx_pack_functions, FunctionsPacking with one task):
the library's colours against golden colourings recorded from the
reference's own src/tools/coloring.cc, against the oracle's restatement of
both colourings and of the subdomain geometry, and against the reference
colouring code itself when it is built here; plus the defining property
(overlapping orbitals never share a colour).  Host code, no GPU."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from mgmol_gb300 import capi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pack_vectors.npz")


def _cases():
    d = np.load(GOLDEN)
    for k in range(int(d["ncases"][0])):
        yield k, d


@pytest.mark.parametrize("rlf", [0, 1])
def test_library_matches_the_golden_colourings(rlf):
    for k, d in _cases():
        n = tuple(int(x) for x in d[f"c{k}_grid"])
        ll = tuple(float(x) for x in d[f"c{k}_ll"])
        sd, ghosts = (int(x) for x in d[f"c{k}_subdiv"])
        col, nc = capi.pack_functions(n, ll, d[f"c{k}_centers"], d[f"c{k}_radii"], sd, rlf,
                                      ghosts)
        assert nc == int(d[f"c{k}_ncolors{rlf}"][0]), k
        assert np.array_equal(col, d[f"c{k}_colors{rlf}"]), k


@pytest.mark.parametrize("rlf", [0, 1])
def test_oracle_matches_the_golden_colourings(rlf):
    for k, d in _cases():
        n = tuple(int(x) for x in d[f"c{k}_grid"])
        ll = tuple(float(x) for x in d[f"c{k}_ll"])
        sd, ghosts = (int(x) for x in d[f"c{k}_subdiv"])
        ov = O.pack_overlap(n, ll, d[f"c{k}_centers"], d[f"c{k}_radii"], sd, ghosts)
        assert np.array_equal(ov, d[f"c{k}_overlap"]), k
        col, nc = O.pack_colors(ov, rlf)
        assert nc == int(d[f"c{k}_ncolors{rlf}"][0]) and np.array_equal(col, d[f"c{k}_colors{rlf}"])


def test_random_layouts_against_restatement_and_reference():
    rng = np.random.default_rng(5)
    n, ll = (64, 48, 40), (22.4, 16.8, 14.0)
    for _ in range(12):
        nf = int(rng.integers(1, 70))
        c = rng.uniform(-5.0, 30.0, size=(nf, 3))   # outside the box too: periodic
        r = rng.uniform(0.5, 4.5, size=nf)
        for sd in (1, 3, 8, 16):
            ov = O.pack_overlap(n, ll, c, r, sd)
            for rlf in (0, 1):
                col, nc = capi.pack_functions(n, ll, c, r, sd, rlf)
                pc, pn = O.pack_colors(ov, rlf)
                assert nc == pn and np.array_equal(col, pc), (nf, sd, rlf)
                ref = O.ref_pack_colors(ov, rlf)
                if ref is not None:
                    assert nc == ref[1] and np.array_equal(col, ref[0]), (nf, sd, rlf)
                # overlapping orbitals never share a colour
                same = col[:, None] == col[None, :]
                assert not np.any(same & (ov > 0) & ~np.eye(nf, dtype=bool))
                assert col.min() == 0 and col.max() == nc - 1


def test_one_subbox_gives_every_orbital_its_own_colour():
    c = np.random.default_rng(1).uniform(0.0, 22.4, size=(20, 3))
    col, nc = capi.pack_functions((64, 64, 64), (22.4,) * 3, c, np.full(20, 0.1), 1)
    assert nc == 20 and sorted(col.tolist()) == list(range(20))


def test_bad_arguments_are_reported():
    with pytest.raises(capi.MgxError):
        capi.pack_functions((64, 64, 64), (22.4,) * 3, np.zeros((2, 3)), np.ones(2), 0)
    with pytest.raises(capi.MgxError):
        capi.pack_functions((64, 64, 64), (22.4,) * 3, np.zeros((2, 3)), np.ones(2), 65)
    col, nc = capi.pack_functions((64, 64, 64), (22.4,) * 3, np.zeros((0, 3)), np.ones(0), 4)
    assert col.size == 0 and nc == 0


def test_adaptor_class_gives_the_library_colours(tmp_path):
    """FunctionsPacking of mgmol_adaptor.h from a C++ program (host only)."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    libdir = os.path.dirname(capi.LIB_PATH)
    capi.load()
    exe = str(tmp_path / "test_pack")
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(root, "mgmol_gb300", "cpp"),
           "-I", os.path.join(cuda, "include"), os.path.join(root, "tests", "cpp", "test_pack.cpp"),
           "-o", exe, "-L", libdir, "-lmgx", f"-Wl,-rpath,{libdir}", "-L",
           os.path.join(cuda, "lib64"), "-lcudart", f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}"]
    subprocess.run(cmd, check=True, capture_output=True)
    rng = np.random.default_rng(9)
    n, ll = (64, 48, 40), (22.4, 16.8, 14.0)
    c = rng.uniform(0.0, 22.0, size=(40, 3))
    r = rng.uniform(1.0, 3.0, size=40).astype(np.float32)
    for rlf in (0, 1):
        text = f"{n[0]} {n[1]} {n[2]} {ll[0]!r} {ll[1]!r} {ll[2]!r} 2 6 {rlf} 40\n" + "".join(
            f"{a!r} {b!r} {d!r} {float(e)!r}\n" for (a, b, d), e in zip(c.tolist(), r))
        out = subprocess.run([exe], input=text, capture_output=True, text=True, check=True).stdout
        vals = [int(x) for x in out.split()]
        col, nc = capi.pack_functions(n, ll, c, r, 6, rlf, ghosts=2)
        assert vals[0] == nc and vals[1:] == col.tolist()
