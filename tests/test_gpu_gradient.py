"""Adjoint gradient of the log-likelihood (emission models).

Checks, on the adjoint workload (80 levels, 6 line species + 2 CIA tables,
11001 wavenumbers, grey cloud with a fixed-bottom, 17 parameters):

* central finite differences (relative step 1e-5, FP64) of the oracle's
  log-likelihood, per component;
* the all-FP64 adjoint (precision mode 1) against the default double-float one;
* chunked evaluation, bit-reproducibility, neglected models, the
  torch.autograd.Function wrapper.

Errors are compared in log-parameter units, x_j dlogL/dx_j (the change of log L
per relative change of the parameter), so every component has the same scale.
The cloud-top pressure enters the reference only through integer layer indices:
its derivative is 0 wherever the indices do not change.
"""

import json
import os

import numpy as np
import pytest

import goldenlib
import oracle
from bear_gb300 import synthetic as syn
from bear_gb300.config import observation_arrays, render_config
from bear_gb300.retrieval import Engine

pytestmark = pytest.mark.gpu

NAME, KIND = "emission_adjoint", "emission"
REPORT = {}


def _record(key, value):
    REPORT[key] = value
    out = os.environ.get("BEAR_GRADIENT_REPORT")
    if out:
        with open(out, "w") as f:
            json.dump(REPORT, f, indent=1)


@pytest.fixture(scope="module")
def case():
    spec = syn.CONFIGS[NAME]
    root = syn.write_tables(spec, goldenlib.TABLE_ROOT)
    text = render_config(syn.global_config(spec, root, KIND), syn.model_config(spec, KIND))
    obs = syn.observations(spec, KIND)
    om0 = oracle.OracleModel(text, [observation_arrays(o) for o in obs])
    _, m, _ = om0.forward(syn.truth_parameters(spec, KIND))
    off, parts = 0, []
    for o in obs:
        parts.append(m[off:off + len(o.data)])
        off += len(o.data)
    syn.attach_data(obs, parts, KIND, spec.seed)
    arrays = [observation_arrays(o) for o in obs]
    e = Engine(text, arrays)
    om = oracle.OracleModel(text, arrays)
    pr = syn.priors(spec, KIND)
    yield spec, e, om, pr
    e.close()


def _points(spec, pr, n, seed):
    cube = np.random.default_rng(seed).uniform(0.05, 0.95, size=(n, len(pr)))
    phys = syn.cube_to_physical(pr, cube)
    phys[0] = syn.truth_parameters(spec, KIND)
    return phys


def _grad(e, phys):
    import torch
    ll, g, ng = e.grad_batch(torch.tensor(phys, device="cuda"))
    return ll.cpu().numpy(), g.cpu().numpy(), ng.cpu().numpy()


def _fd(om, x, j, rel):
    h = rel * abs(x[j])
    xp, xm = x.copy(), x.copy()
    xp[j] += h
    xm[j] -= h
    return (om.loglike(xp) - om.loglike(xm)) / (2 * h)


def test_gradient_against_oracle_finite_differences(case):
    """Central differences of the oracle with relative steps 1e-5 and 5e-6,
    Richardson-extrapolated (the likelihood of 1%-error data is strongly curved:
    a single 1e-5 step leaves ~1e-5 relative truncation error in d/d log g)."""
    spec, e, om, pr = case
    phys = _points(spec, pr, 3, 11)
    ll, g, ng = _grad(e, phys)
    names = [p.description for p in pr]
    worst, worst_raw = {}, {}
    for i in range(len(phys)):
        assert not ng[i]
        x = phys[i]
        assert abs(ll[i] - om.loglike(x)) <= 1e-8 + 1e-12 * abs(ll[i])
        d1 = np.array([_fd(om, x, j, 1e-5) for j in range(len(x))])
        d2 = np.array([_fd(om, x, j, 5e-6) for j in range(len(x))])
        fd = (4 * d2 - d1) / 3
        sa, sf, s1 = x * g[i], x * fd, x * d1  # log-parameter units
        scale = np.max(np.abs(sf))
        for j, nm in enumerate(names):
            err = abs(sa[j] - sf[j])
            big = abs(sf[j]) > 1e-6 * scale
            worst[nm] = max(worst.get(nm, 0.0), err / abs(sf[j]) if big else err / scale)
            worst_raw[nm] = max(worst_raw.get(nm, 0.0), abs(sa[j] - s1[j]) / max(abs(s1[j]), 1e-300))
            if nm == "cloud top pressure":
                assert g[i][j] == 0.0 and fd[j] == 0.0
                continue
            # FD noise: ~1e-15 |log L| per evaluation over a 1e-5 step, amplified by the extrapolation
            tol = 1e-6 * abs(sf[j]) + 1e-8 * scale + 2e-10 * abs(ll[i]) / 1e-5
            assert err <= tol, (i, nm, sa[j], sf[j], err, tol)
    _record("fd_richardson_vs_adjoint_rel_err_per_component", worst)
    _record("fd_1e-5_vs_adjoint_rel_err_per_component", worst_raw)


def test_double_float_adjoint_against_fp64_adjoint(case):
    spec, e, om, pr = case
    phys = _points(spec, pr, 24, 12)
    ll0, g0, _ = _grad(e, phys)
    e.set_precision(1)
    try:
        ll1, g1, _ = _grad(e, phys)
    finally:
        e.set_precision(0)
    s0, s1 = phys * g0, phys * g1
    scale = np.abs(s1).max(axis=1, keepdims=True)
    err = np.abs(s0 - s1) / scale
    _record("df_vs_fp64_adjoint_max_rel", float(err.max()))
    assert err.max() < 1e-9
    assert np.all(np.abs(ll0 - ll1) <= 1e-8 + 1e-12 * np.abs(ll1))


def test_gradient_loglike_equals_batched_forward(case):
    import torch
    spec, e, om, pr = case
    phys = _points(spec, pr, 40, 13)
    ll, g, ng = _grad(e, phys)
    ll2, ng2 = e.loglike_batch(torch.tensor(phys, device="cuda"))
    assert np.array_equal(ll, ll2.cpu().numpy())
    assert np.array_equal(ng, ng2.cpu().numpy())


def test_chunked_gradient_is_bit_identical(case):
    spec, e, om, pr = case
    phys = _points(spec, pr, 20, 14)
    ll0, g0, _ = _grad(e, phys)
    ll0b, g0b, _ = _grad(e, phys)
    assert np.array_equal(g0, g0b) and np.array_equal(ll0, ll0b)  # reproducible
    e.set_gradient_memory(3 * 80 * 2 * 11001 * 8 + (1 << 20))     # about 3 evaluations per chunk
    try:
        ll1, g1, _ = _grad(e, phys)
    finally:
        e.set_gradient_memory(0)
    assert np.array_equal(ll0, ll1)
    assert np.array_equal(g0, g1)


def test_neglected_model_has_zero_gradient(case):
    spec, e, om, pr = case
    phys = _points(spec, pr, 4, 15)
    ti = [p.description for p in pr].index("T0")
    phys[1, ti] = 20.0  # knots below the 50 K clamp -> neglected
    ll, g, ng = _grad(e, phys)
    assert ng[1] and ll[1] == -1e30
    assert np.all(g[1] == 0.0)
    assert not ng[0] and np.any(g[0] != 0.0)


def test_autograd_function(case):
    import torch
    from bear_gb300.autograd import log_likelihood
    spec, e, om, pr = case
    phys = _points(spec, pr, 6, 16)
    P = torch.tensor(phys, device="cuda", requires_grad=True)
    w = torch.linspace(0.5, 1.5, len(phys), dtype=torch.float64, device="cuda")
    (w * log_likelihood(e, P)).sum().backward()
    _, g, _ = _grad(e, phys)
    assert np.array_equal(P.grad.cpu().numpy(), w.cpu().numpy()[:, None] * g)
    with torch.no_grad():
        ll = log_likelihood(e, P.detach())
    ll2, _ = e.loglike_batch(P.detach())
    assert torch.equal(ll, ll2)
