"""Adjoint gradient of emission models with the non-grey clouds.

The power-law cloud (PowerLawCloudModel, src/cloud_model/power_law_cloud_model.cpp:69-121)
and the KH cloud (KHCloudModel, src/cloud_model/kh_cloud_model.cpp:69-133) scale the cloud
layers' optical depth by a wavelength factor of their shape parameters (the power-law
exponent; q0, a0 and the particle size). The adjoint weights each level's cloud sink by that
factor and sums the layers' cloud depths times the factor's derivatives, so every
continuous parameter, the shape parameters included, is checked against central
differences (relative steps 1e-5 and 5e-6, Richardson-extrapolated) of the FP64 oracle;
the cloud-top pressure and bottom factor place the cloud on whole layers and have a zero
gradient, as for the grey cloud.

Cases: the power-law golden set (50 levels, 3 line species + 2 CIA, H2 Rayleigh, 16
parameters) at its three parameter vectors, and the same atmosphere with the KH cloud
(bottom from the scale height) at one point.
"""

import os

import numpy as np
import pytest

import goldenlib
import oracle
from bear_gb300.retrieval import Engine

pytestmark = pytest.mark.gpu


def _fd(f, x, j, rel):
    h = rel * abs(x[j])
    xp, xm = x.copy(), x.copy()
    xp[j] += h
    xm[j] -= h
    return (f(xp) - f(xm)) / (2 * h)


def _check(e, om, phys, discrete):
    import torch
    ll, g, ng = e.grad_batch(torch.tensor(phys, device="cuda"))
    ll, g, ng = ll.cpu().numpy(), g.cpu().numpy(), ng.cpu().numpy()
    for i in range(len(phys)):
        assert not ng[i]
        x = phys[i]
        assert abs(ll[i] - om.loglike(x)) <= 1e-8 + 1e-12 * abs(ll[i])
        fd = np.array([(4 * _fd(om.loglike, x, j, 5e-6) - _fd(om.loglike, x, j, 1e-5)) / 3 if j not in discrete
                       else 0.0 for j in range(len(x))])
        sa, sf = x * g[i], x * fd
        scale = np.max(np.abs(sf))
        for j in range(len(x)):
            if j in discrete:
                assert g[i][j] == 0.0, (i, j, g[i][j])
                continue
            err = abs(sa[j] - sf[j])
            tol = 1e-6 * abs(sf[j]) + 1e-8 * scale + 2e-10 * abs(ll[i]) / 1e-5
            assert err <= tol, (i, j, sa[j], sf[j], err, tol)


def test_power_law_cloud_gradient():
    c = goldenlib.Case(os.path.join(goldenlib.GOLDEN_DIR, "emission_powerlaw_cloud.npz"))
    text, obs = c.config_text(), c.observations()
    assert "cloud power_law" in text
    e = Engine(text, obs)
    om = oracle.OracleModel(text, obs)
    try:
        phys = np.array(c.params, dtype=np.float64)
        # tau, exponent, top pressure, bottom factor: the last two place the cloud layers
        _check(e, om, phys, discrete=(14, 15))
    finally:
        om.close()
        e.close()


def test_kh_cloud_gradient():
    c = goldenlib.Case(os.path.join(goldenlib.GOLDEN_DIR, "emission_powerlaw_cloud.npz"))
    text = c.config_text()
    lines = [("cloud KHnongrey 1.0 fb" if ln.startswith("cloud power_law") else ln) for ln in text.splitlines()]
    text = "\n".join(lines) + "\n"
    obs = c.observations()
    e = Engine(text, obs)
    om = oracle.OracleModel(text, obs)
    try:
        base = np.array(c.params[0], dtype=np.float64)
        # tau, q0, a0, particle size (micron), top pressure (bottom from the scale height)
        phys = np.concatenate([base[:12], [3.0, 8.0, 3.5, 0.6, 0.3]])[None, :]
        assert phys.shape[1] == e.P
        _check(e, om, phys, discrete=(16,))
    finally:
        om.close()
        e.close()
