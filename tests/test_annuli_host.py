"""Transit depth with A impact parameters per layer (``transmission_annuli A``, not in the
reference) in the FP64 oracle: A = 1 is the reference's tangent-ray formula (the golden
spectra), and the spectra converge as A grows. The engine is checked against these oracle
spectra in test_gpu_annuli.py."""

import os

import pytest

import goldenlib
import oracle
from bear_gb300.config import TransmissionModelConfig, render_config
from bear_gb300 import synthetic as syn


@pytest.fixture(scope="module")
def case():
    return goldenlib.Case(os.path.join(goldenlib.GOLDEN_DIR, "transmission_kh_cloud.npz"))


def _model(c, annuli):
    text = c.config_text() + (f"transmission_annuli {annuli}\n" if annuli is not None else "")
    return oracle.OracleModel(text, c.observations())


def test_one_annulus_is_the_reference_formula(case):
    om = _model(case, 1)
    for i, p in enumerate(case.params):
        spec, obs, _ = om.forward(p)
        assert goldenlib.rel_err(obs, case.arrays["ref_obs"][i]) < 1e-12
        assert abs(om.loglike(p) - case.arrays["ref_loglike"][i]) <= 1e-8


def test_spectra_converge_with_annuli(case):
    p = case.params[0]
    spectra = {a: _model(case, a).forward(p)[0] for a in (1, 2, 5, 10, 20, 40)}
    d = [goldenlib.rel_err(spectra[a], spectra[40]) for a in (1, 2, 5, 10, 20)]
    assert all(x > y for x, y in zip(d, d[1:])), d
    assert d[3] < 1e-3, d          # 10 rays per layer: within 0.1 % of 40
    assert d[0] > d[3] * 2, d      # the finer rays change the spectrum


def test_annuli_out_of_range_is_rejected(case):
    with pytest.raises(Exception):
        _model(case, 65)


def test_config_renders_annuli():
    spec = syn.CONFIGS["transmission_plain"]
    mc = syn.model_config(spec, "transmission")
    assert isinstance(mc, TransmissionModelConfig)
    text = render_config(syn.global_config(spec, "/tmp/tables/", "transmission"), mc)
    assert "transmission_annuli" not in text
    mc.transmission_annuli = 10
    text = render_config(syn.global_config(spec, "/tmp/tables/", "transmission"), mc)
    assert "transmission_annuli 10\n" in text
