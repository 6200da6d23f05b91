"""Contribution functions (bear_contribution_functions) against the FP64 oracle's
restatement of the reference's contribution-function kernel and post-process binning,
on the emission, H- emission, power-law-cloud emission and blackbody-eclipse golden
cases. The engine's opacities are double-float, so the bound is 1e-9 relative (the
reference itself stores its opacities as floats)."""

import numpy as np
import pytest

import goldenlib
import oracle
from bear_gb300 import _lib
from bear_gb300.retrieval import Engine

pytestmark = pytest.mark.gpu

NAMES = ["emission_plain", "emission_hminus", "emission_powerlaw_cloud", "eclipse_blackbody"]


@pytest.mark.parametrize("name", NAMES)
def test_contribution_functions_against_oracle(name):
    c = goldenlib.Case(goldenlib.GOLDEN_DIR + f"/{name}.npz")
    e = Engine(c.config_text(), c.observations())
    om = oracle.OracleModel(c.config_text(), c.observations())
    L = e.table_info()["levels"]
    try:
        for p in c.params[:2]:
            bins, hr = e.contribution_functions(p)
            ref_hr, ref_bins = om.contribution(p, L)
            assert np.all(hr[0] == 0.0) and np.all(bins[0] == 0.0)
            scale = np.abs(ref_hr).max()
            assert np.all(np.abs(hr - ref_hr) <= 1e-9 * np.abs(ref_hr) + 1e-13 * scale)
            bscale = np.abs(ref_bins).max()
            assert np.all(np.abs(bins - ref_bins) <= 1e-9 * np.abs(ref_bins) + 1e-13 * bscale)
            assert np.all(hr >= 0.0)
        e.set_precision(1)
        bins64, hr64 = e.contribution_functions(c.params[0])
        ref_hr, ref_bins = om.contribution(c.params[0], L)
        assert np.all(np.abs(hr64 - ref_hr) <= 1e-11 * np.abs(ref_hr) + 1e-14 * np.abs(ref_hr).max())
    finally:
        e.close()


def test_contribution_functions_rejected_for_transmission():
    c = goldenlib.Case(goldenlib.GOLDEN_DIR + "/transmission_plain.npz")
    e = Engine(c.config_text(), c.observations())
    try:
        with pytest.raises(_lib.EngineError) as ei:
            e.contribution_functions(c.params[0])
        assert ei.value.code == 4
    finally:
        e.close()
