"""Localization regions of one task (mgx_regions_move_to,
mgx_regions_update_radii) against the oracle's restatement of
LocalizationRegions::moveTo / updateRadii / getMeanRadius: bit for bit on
seeded and crafted cases (periodic wrap, the 1-bohr cap)."""
import numpy as np

import oracle as O
from mgmol_gb300 import capi

CELL = (22.4, 16.8, 14.0)


def test_move_to_matches_the_oracle():
    rng = np.random.default_rng(3)
    c = rng.uniform(0.0, 1.0, size=(200, 3)) * np.asarray(CELL)
    # small moves, long moves (capped), and targets across the periodic faces
    t = c + rng.normal(0.0, 0.3, size=c.shape)
    t[50:100] += rng.normal(0.0, 3.0, size=(50, 3))
    t[100:150] = t[100:150] + np.asarray(CELL) * rng.integers(-2, 3, size=(50, 3))
    got, mx = capi.regions_move_to(c, t, CELL)
    ref, rmx = O.regions_move_to(c, t, CELL)
    assert np.array_equal(got, ref) and mx == rmx
    step = got - c
    # the cap divides by the FP32 length, so a capped step is 1 to FP32 rounding
    assert np.all(np.linalg.norm(step, axis=1) <= 1.0 + 1e-6)


def test_move_to_reaches_near_targets_and_caps_far_ones():
    c = np.array([[1.0, 1.0, 1.0], [21.9, 0.2, 13.9], [5.0, 5.0, 5.0]])
    t = np.array([[1.3, 0.8, 1.1], [0.1, 16.6, 0.1], [9.0, 5.0, 5.0]])
    got, mx = capi.regions_move_to(c, t, CELL)
    assert np.allclose(got[0], t[0])
    # across the faces: the short way round, 0.6 / -0.4 / 0.2 bohr
    assert np.allclose(got[1], c[1] + [0.6, -0.4, 0.2])
    assert np.allclose(got[2], [6.0, 5.0, 5.0]) and abs(mx - 4.0) < 1e-6


def test_update_radii_matches_the_oracle():
    sp = np.random.default_rng(4).uniform(0.5, 3.0, size=77)
    r, mean = capi.regions_update_radii(sp, 2.5)
    rr, rmean = O.regions_update_radii(sp, 2.5)
    assert np.array_equal(r, rr)
    assert abs(mean - rmean) <= 1e-6 * rmean
