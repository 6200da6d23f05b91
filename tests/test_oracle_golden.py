"""The C oracle against outputs of the reference's own CPU path (golden cases)."""

import os

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


@pytest.mark.parametrize("name", ["emission_edges", "eclipse_blackbody"])
def test_variable_gravity_is_ignored_by_emission_models(name):
    """The reference's emission and secondary-eclipse models build their structure with
    constant gravity whatever the config says (EmissionModel::calcAtmosphereStructure
    src/forward_model/emission/emission.cpp:178-185, OccultationModel::calcAtmosphereStructure
    src/forward_model/secondary_eclipse/secondary_eclipse.cpp:165-172): the oracle gives
    the same log L with the variable-gravity key on."""
    c = goldenlib.Case(os.path.join(goldenlib.GOLDEN_DIR, name + ".npz"))
    obs = c.observations()
    base = oracle.OracleModel(c.config_text(), obs)
    varg = oracle.OracleModel(c.config_text() + "variable_gravity 1\n", obs)
    try:
        for p in c.params[:2]:
            assert varg.loglike(p) == base.loglike(p)
    finally:
        base.close()
        varg.close()
