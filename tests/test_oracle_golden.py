"""The C oracle against outputs of the reference's own CPU path (golden cases)."""

import numpy as np
import pytest

import goldenlib
import oracle

CASES = goldenlib.golden_cases()


@pytest.fixture(scope="module", params=CASES, ids=lambda p: p.split("/")[-1][:-4])
def case(request):
    c = goldenlib.Case(request.param)
    return c, oracle.OracleModel(c.config_text(), c.observations())


def test_grid_and_setup(case):
    c, om = case
    assert np.array_equal(om.grid(), c.arrays["ref_grid"])
    for k in range(len(c.observations())):
        assert om.obs_setup(k) == c.setup(k)


def test_forward_and_loglike(case):
    c, om = case
    rows = list(c.arrays["spectrum_rows"])
    for i, p in enumerate(c.params):
        spec, obs, neg = om.forward(p)
        assert neg == bool(c.arrays["ref_neglect"][i])
        assert goldenlib.rel_err(obs, c.arrays["ref_obs"][i]) < 1e-12
        if i in rows:
            assert goldenlib.rel_err(spec, c.arrays["ref_spectrum"][rows.index(i)]) < 1e-12
        ll = om.loglike(p)
        ref = c.arrays["ref_loglike"][i]
        assert abs(ll - ref) <= 1e-8 + 1e-14 * abs(ref), (i, ll, ref)
