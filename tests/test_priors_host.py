"""Host mirror of the reference's prior transforms (no GPU): uniform, log-uniform,
Gaussian, delta and linked priors with units, against the formulas of
src/retrieval/prior_types.h:89-256, and the linked-prior checks of
src/retrieval/priors.cpp:246-280."""

import math

import numpy as np
import pytest

from bear_gb300.config import Prior
from bear_gb300.retrieval import UNITS, Priors


def _priors():
    return [Prior("uniform", "log g", [5.5, 4.5]),           # reversed bounds are swapped
            Prior("uniform", "R", [0.8, 1.6], "Rj"),
            Prior("log_uniform", "H2O", [1e-8, 1e-2]),
            Prior("gaussian", "d", [10.0, 0.5], "pc"),
            Prior("delta", "f", [1.0]),
            Prior("linked", "R2", [2]),                      # follows parameter 2 (1-based), no unit
            Prior("log_uniform", "CO", [1e-3, 1e-9])]


def test_host_transform_matches_the_reference_formulas():
    pr = Priors(_priors())
    rng = np.random.default_rng(3)
    cube = rng.uniform(size=(50, 7))
    batch = pr.cube_to_physical_batch(cube)
    for row, c in zip(batch, cube):
        par = pr.cube_to_parameters(list(c))
        phys = pr.to_physical(par)
        assert np.allclose(row, phys, rtol=1e-15, atol=0)
        assert row[0] == 4.5 + c[0] * 1.0
        assert row[1] == (0.8 + c[1] * (1.6 - 0.8)) * UNITS["Rj"]
        assert math.isclose(row[2], 10 ** (-8 + c[2] * 6), rel_tol=1e-15)
        from scipy.special import erfinv
        assert math.isclose(row[3], (10 + 0.5 * math.sqrt(2) * erfinv(2 * c[3] - 1)) * UNITS["pc"], rel_tol=1e-15)
        assert row[4] == 1.0
        assert row[5] == 0.8 + c[1] * (1.6 - 0.8)           # linked: parameter 2's value, no unit
        assert math.isclose(row[6], 10 ** (-9 + c[6] * 6), rel_tol=1e-15)


def test_linked_prior_errors():
    with pytest.raises(ValueError, match="wrong index"):
        Priors([Prior("uniform", "a", [0, 1]), Prior("linked", "b", [3])])
    with pytest.raises(ValueError, match="another linked"):
        Priors([Prior("uniform", "a", [0, 1]), Prior("linked", "b", [1]), Prior("linked", "c", [2])])
    with pytest.raises(ValueError, match="unknown"):
        Priors([Prior("cauchy", "a", [0, 1])])


def _golden_priors():
    import json
    import os

    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "priors.npz"))
    meta = json.loads(bytes(z["meta"]).decode())
    return [Prior(t, d, p, u) for t, d, p, u in meta["priors"]], z


def test_host_transform_matches_the_reference_binary():
    """Against Retrieval::convertCubeParameters of the reference itself
    (tests/golden/priors.npz, made by tests/golden/make_golden.py priors): uniform,
    log-uniform, delta and linked priors with every unit; the Gaussian prior is pinned only
    to the published erfinv formula above, because the reference takes erf_inv from
    Boost.Math, which is not available to build it here."""
    pr, z = _golden_priors()
    host = Priors(pr).cube_to_physical_batch(z["cube"])
    ref = z["ref_physical"]
    err = np.abs(host - ref) / np.maximum(np.abs(ref), 1e-300)
    assert err.max() <= 4e-16, err.max()
