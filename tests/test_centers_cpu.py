"""The oracle of the orbital centres (SpreadsAndCenters with
SinCosOps::computeDiag): its position tables against golden tables recorded
from the reference's own pb::Grid, and against that code itself when it is
built here; the centre and spread of a Gaussian from the oracle's sums."""
import os

import numpy as np

import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "centers_vectors.npz")


def test_tables_match_the_reference_bit_for_bit():
    d = np.load(GOLDEN)
    for k in range(int(d["ngrids"][0])):
        n = tuple(int(x) for x in d[f"g{k}_n"])
        ll = tuple(float(x) for x in d[f"g{k}_ll"])
        assert np.array_equal(O.sincos_tables(n, ll), d[f"g{k}_tables"]), n
        ref = O.sincos_tables(n, ll, ref=True)
        if ref is not None:
            assert np.array_equal(ref, d[f"g{k}_tables"]), n


def test_gaussian_centre_and_spread():
    n, ll = (48, 40, 36), (16.8, 14.0, 12.6)
    h = [ll[i] / n[i] for i in range(3)]
    c = np.array([3.3, 12.9, 0.4])  # near a face: periodic images matter
    sig = 1.1
    ax = [np.arange(n[i]) * h[i] for i in range(3)]
    d2 = 0.
    for i in range(3):
        di = ax[i] - c[i]
        di = di - ll[i] * np.round(di / ll[i])
        shape = [1, 1, 1]
        shape[i] = n[i]
        d2 = d2 + (di ** 2).reshape(shape)
    psi = np.exp(-d2 / (2 * sig * sig)).reshape(1, -1)
    a = O.sincos_diag(n, ll, psi)
    x, spread = O.centers_spreads(ll, a)
    assert np.max(np.abs(x[0] - c)) < 1e-6
    # |psi|^2 is a Gaussian of variance s2 = sig^2 / 2 per direction, whose
    # first Fourier coefficient has modulus exp(-k^2 s2 / 2), k = 2 pi / L:
    # the spread^2 is sum (1 - exp(-k^2 s2)) / k^2
    s2 = sig * sig / 2
    k = 2 * np.pi / np.asarray(ll)
    expect = np.sqrt(np.sum((1 - np.exp(-k * k * s2)) / (k * k)))
    assert abs(spread[0] - expect) < 1e-6
    # normalized form: the same elements up to the norm
    norm = np.sum(psi ** 2) * h[0] * h[1] * h[2]
    assert np.allclose(O.sincos_diag(n, ll, psi / np.sqrt(norm), normalized=True), a, rtol=1e-12)
