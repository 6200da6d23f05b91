"""H- continuum (bound-free + free-free) in the batched emission workload (80 levels,
6 line species, 11001 points at 1 cm^-1 from 0.8 um, H, H- and e- in the chemistry)
against the FP64 oracle, the double-float path against the FP64 path, and the emission
gradient with the H- continuum against the oracle's differences, and the transmission
gradient with the H- continuum and with the KH cloud likewise."""

import dataclasses

import numpy as np
import pytest

import goldenlib
import oracle
from bear_gb300 import _lib
from bear_gb300 import synthetic as syn
from bear_gb300.config import observation_arrays, render_config
from bear_gb300.retrieval import Engine

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    spec = syn.CONFIGS["emission_batched"]
    root = syn.write_tables(spec, goldenlib.TABLE_ROOT)
    text = render_config(syn.global_config(spec, root, "emission"), syn.model_config(spec, "emission"))
    chem = "chemistry iso " + " ".join(spec.species) + "\n"
    assert chem in text
    text = text.replace(chem, chem[:-1] + " H H- e-\n") + "opacity H-\n"
    obs = syn.observations(spec, "emission")
    pr = syn.priors(spec, "emission")
    ns = len(spec.species)
    truth = np.concatenate([syn.truth_parameters(spec, "emission")[:3 + ns], [1e-3, 1e-9, 1e-6],
                            syn.truth_parameters(spec, "emission")[3 + ns:]])
    om0 = oracle.OracleModel(text, [observation_arrays(o) for o in obs])
    _, m, _ = om0.forward(truth)
    off, parts = 0, []
    for o in obs:
        parts.append(m[off:off + len(o.data)])
        off += len(o.data)
    syn.attach_data(obs, parts, "emission", spec.seed)
    arrays = [observation_arrays(o) for o in obs]
    e = Engine(text, arrays)
    yield e, oracle.OracleModel(text, arrays), truth, ns
    e.close()


def _points(truth, ns, n, seed):
    rng = np.random.default_rng(seed)
    p = np.tile(truth, (n, 1))
    p[:, 3 + ns:6 + ns] = 10.0 ** rng.uniform([-6, -12, -9], [-2, -7, -4], size=(n, 3))  # H, H-, e-
    p[:, 6 + ns] = rng.uniform(1800.0, 3200.0, n)                                        # T0
    p[1, 4 + ns] = 0.0                                                                   # no H-
    return p


def test_hminus_batch_against_oracle(case):
    import torch
    e, om, truth, ns = case
    phys = _points(truth, ns, 16, 1)
    phys[0] = truth
    ll, ng = e.loglike_batch(torch.tensor(phys, device="cuda"))
    ll = ll.cpu().numpy()
    for i in range(6):
        ref = om.loglike(phys[i])
        _, obs_ref, neg_ref = om.forward(phys[i])
        assert bool(ng[i]) == neg_ref
        assert abs(ll[i] - ref) <= 1e-8 + 1e-12 * abs(ref), (i, ll[i], ref)
        spec, obs, _ = e.compute_model(phys[i])
        assert goldenlib.rel_err(obs, obs_ref) < 1e-6


def test_hminus_double_float_against_fp64(case):
    import torch
    e, om, truth, ns = case
    P = torch.tensor(_points(truth, ns, 32, 2), device="cuda")
    ll_df, _ = e.loglike_batch(P)
    e.set_precision(1)
    try:
        ll_64, _ = e.loglike_batch(P)
    finally:
        e.set_precision(0)
    d = (ll_df - ll_64).abs().cpu().numpy()
    assert np.all(d <= 1e-8 + 1e-12 * ll_64.abs().cpu().numpy()), d.max()


def _fd(f, x, j, rel):
    h = rel * abs(x[j])
    xp, xm = x.copy(), x.copy()
    xp[j] += h
    xm[j] -= h
    return (f(xp) - f(xm)) / (2 * h)


def test_hminus_gradient_against_oracle(case):
    """The emission adjoint with the H- continuum: the level sinks of its seven
    coefficients (sum over wavenumbers of d log L / d kappa times the coefficient rows)
    mapped through the coefficients' tangents (n(H-), n(e-) k T n(H) (5040/T)^((i+1)/2)),
    every parameter against the oracle's Richardson central differences; at the point
    without H- the free-free terms are held at zero."""
    import torch
    e, om, truth, ns = case
    phys = _points(truth, ns, 3, 7)
    phys[0] = truth
    ll, g, ng = e.grad_batch(torch.tensor(phys, device="cuda"))
    ll, g = ll.cpu().numpy(), g.cpu().numpy()
    for i in range(len(phys)):
        assert not ng[i]
        x = phys[i]
        assert abs(ll[i] - om.loglike(x)) <= 1e-8 + 1e-12 * abs(ll[i])
        fd = np.zeros(len(x))
        for j in range(len(x)):
            if x[j] == 0.0:
                continue  # a zero H- abundance: no relative step
            fd[j] = (4 * _fd(om.loglike, x, j, 5e-6) - _fd(om.loglike, x, j, 1e-5)) / 3
        sa, sf = x * g[i], x * fd
        scale = np.max(np.abs(sf))
        for j in range(len(x)):
            err = abs(sa[j] - sf[j])
            tol = 1e-6 * abs(sf[j]) + 1e-8 * scale + 2e-10 * abs(ll[i]) / 1e-5
            assert err <= tol, (i, j, sa[j], sf[j], err, tol)


def test_hminus_transmission_gradient_against_oracle():
    """The transmission adjoint with the H- continuum (its seven coefficients are linear
    opacity terms after the Rayleigh rows, so the level sinks already cover them; the
    per-evaluation tangents map them), against the oracle's Richardson differences with
    the tau > 10 cut-off disabled in both, at the golden points (one without H-)."""
    import torch
    c = [goldenlib.Case(p) for p in goldenlib.golden_cases() if p.endswith("transmission_hminus.npz")][0]
    text = c.config_text().replace("variable_gravity 1", "variable_gravity 0")
    obs = c.observations()
    e = Engine(text, obs)
    om = oracle.OracleModel(text, obs)
    e.set_tau_cutoff(float("inf"))
    om.set_tau_cutoff(float("inf"))
    try:
        phys = np.array(c.params, dtype=np.float64)
        ll, g, ng = e.grad_batch(torch.tensor(phys, device="cuda"))
        ll, g = ll.cpu().numpy(), g.cpu().numpy()
        for i in range(len(phys)):
            assert not ng[i]
            x = phys[i]
            assert abs(ll[i] - om.loglike(x)) <= 1e-8 + 1e-12 * abs(ll[i])
            fd = np.zeros(len(x))
            for j in range(len(x)):
                if x[j] != 0.0:
                    fd[j] = (4 * _fd(om.loglike, x, j, 5e-6) - _fd(om.loglike, x, j, 1e-5)) / 3
            sa, sf = x * g[i], x * fd
            scale = np.max(np.abs(sf))
            for j in range(len(x)):
                err = abs(sa[j] - sf[j])
                tol = 1e-6 * abs(sf[j]) + 1e-8 * scale + 2e-10 * abs(ll[i]) / 1e-5
                assert err <= tol, (i, j, sa[j], sf[j], err, tol)
    finally:
        e.set_tau_cutoff(10.0)
        om.close()
        e.close()


def test_transmission_kh_cloud_gradient_against_oracle():
    """The transmission adjoint with the KH cloud: the level's cloud sink weighted by the
    wavelength factor, and the sums along q0, a0 and the particle size (the factor's
    derivatives per wavenumber, tr_cloud_shape_kernel), against the oracle's Richardson
    differences with the tau > 10 cut-off disabled; the cloud-top pressure places whole
    layers (zero gradient). The golden set's first point is left out: there the cloud bottom
    (one scale height below the top) moves by a level within the difference step in T, and
    the differences of the grey cloud at that point miss the adjoint by the same 2 %."""
    import torch
    c = [goldenlib.Case(p) for p in goldenlib.golden_cases() if p.endswith("transmission_kh_cloud.npz")][0]
    text = c.config_text().replace("variable_gravity 1", "variable_gravity 0")
    obs = c.observations()
    e = Engine(text, obs)
    om = oracle.OracleModel(text, obs)
    e.set_tau_cutoff(float("inf"))
    om.set_tau_cutoff(float("inf"))
    try:
        phys = np.array(c.params[1:], dtype=np.float64)
        top = phys.shape[1] - 1  # cloud-top pressure (the bottom follows the scale height)
        ll, g, ng = e.grad_batch(torch.tensor(phys, device="cuda"))
        ll, g = ll.cpu().numpy(), g.cpu().numpy()
        for i in range(len(phys)):
            assert not ng[i]
            x = phys[i]
            assert abs(ll[i] - om.loglike(x)) <= 1e-8 + 1e-12 * abs(ll[i])
            assert g[i][top] == 0.0
            fd = np.zeros(len(x))
            for j in range(len(x)):
                if x[j] != 0.0 and j != top:
                    fd[j] = (4 * _fd(om.loglike, x, j, 5e-6) - _fd(om.loglike, x, j, 1e-5)) / 3
            sa, sf = x * g[i], x * fd
            scale = np.max(np.abs(sf))
            for j in range(len(x)):
                if j == top:
                    continue
                err = abs(sa[j] - sf[j])
                tol = 1e-6 * abs(sf[j]) + 1e-8 * scale + 2e-10 * abs(ll[i]) / 1e-5
                assert err <= tol, (i, j, sa[j], sf[j], err, tol)
    finally:
        e.set_tau_cutoff(10.0)
        om.close()
        e.close()
