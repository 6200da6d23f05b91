"""Adjoint gradient of the log-likelihood of transmission models.

Workload: 100 levels, 8 line species + 2 CIA + H2/He Rayleigh, 33976 points,
grey cloud, 300 transit-depth bins; 14 parameters.

The reference's tau > 10 cut-off of the tangent-ray sums makes log L a step
function of the parameters wherever a ray's partial sum crosses 10, so central
differences of the model with the cut-off are dominated by those steps. The
adjoint (which holds the cut-off indices fixed) is therefore checked against
central differences (relative steps 1e-5 and 5e-6, Richardson-extrapolated) of
the FP64 oracle and of the engine with the cut-off disabled, where the model is
smooth; with the cut-off, the stellar-radius component (depth ~ 1/R_s^2, no
cut-off dependence) is checked, and log L must equal the batched forward pass.
"""

import json
import os

import numpy as np
import pytest

import goldenlib
import oracle
from bear_gb300 import _lib
from bear_gb300 import synthetic as syn
from bear_gb300.config import observation_arrays, render_config
from bear_gb300.retrieval import Engine

pytestmark = pytest.mark.gpu

NAME, KIND = "transmission_plain", "transmission"
REPORT = {}


def _record(key, value):
    REPORT[key] = value
    out = os.environ.get("BEAR_GRADIENT_REPORT_TR")
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
    yield spec, e, om, syn.priors(spec, KIND)
    e.close()


def _points(spec, pr, n, seed):
    phys = syn.cube_to_physical(pr, np.random.default_rng(seed).uniform(0.05, 0.95, size=(n, len(pr))))
    phys[0] = syn.truth_parameters(spec, KIND)
    return phys


def _grad(e, phys):
    import torch
    ll, g, ng = e.grad_batch(torch.tensor(phys, device="cuda"))
    return ll.cpu().numpy(), g.cpu().numpy(), ng.cpu().numpy()


def _fd(f, x, j, rel):
    h = rel * abs(x[j])
    xp, xm = x.copy(), x.copy()
    xp[j] += h
    xm[j] -= h
    return (f(xp) - f(xm)) / (2 * h)


def test_transmission_gradient_against_oracle_without_cutoff(case):
    spec, e, om, pr = case
    names = [p.description for p in pr]
    e.set_tau_cutoff(float("inf"))
    om.set_tau_cutoff(float("inf"))
    try:
        phys = _points(spec, pr, 2, 21)
        ll, g, ng = _grad(e, phys)
        worst = {}
        for i in range(len(phys)):
            assert not ng[i]
            x = phys[i]
            assert abs(ll[i] - om.loglike(x)) <= 1e-8 + 1e-12 * abs(ll[i])
            d1 = np.array([_fd(om.loglike, x, j, 1e-5) for j in range(len(x))])
            d2 = np.array([_fd(om.loglike, x, j, 5e-6) for j in range(len(x))])
            fd = (4 * d2 - d1) / 3
            sa, sf = x * g[i], x * fd
            scale = np.max(np.abs(sf))
            for j, nm in enumerate(names):
                err = abs(sa[j] - sf[j])
                big = abs(sf[j]) > 1e-6 * scale
                worst[nm] = max(worst.get(nm, 0.0), err / abs(sf[j]) if big else err / scale)
                if nm == "cloud top pressure":
                    assert g[i][j] == 0.0
                    continue
                tol = 1e-6 * abs(sf[j]) + 1e-8 * scale + 2e-10 * abs(ll[i]) / 1e-5
                assert err <= tol, (i, nm, sa[j], sf[j], err, tol)
        _record("no_cutoff_fd_richardson_vs_adjoint_rel_err_per_component", worst)
    finally:
        e.set_tau_cutoff(10.0)
        om.set_tau_cutoff(10.0)


def test_transmission_gradient_with_cutoff(case):
    import torch
    spec, e, om, pr = case
    names = [p.description for p in pr]
    phys = _points(spec, pr, 8, 22)
    ll, g, ng = _grad(e, phys)
    ll2, ng2 = e.loglike_batch(torch.tensor(phys, device="cuda"))
    assert np.array_equal(ll, ll2.cpu().numpy()) and np.array_equal(ng, ng2.cpu().numpy())
    assert np.all(np.isfinite(g))
    # the stellar radius scales every depth by 1 / R_s^2 and moves no cut-off
    js = names.index("R_s")
    for i in range(3):
        x = phys[i]
        f = lambda p: float(e.loglike_batch(torch.tensor(p[None, :], device="cuda"))[0][0])
        fd = (4 * _fd(f, x, js, 5e-6) - _fd(f, x, js, 1e-5)) / 3
        assert abs(g[i][js] - fd) <= 1e-7 * abs(fd), (i, g[i][js], fd)


def test_transmission_gradient_chunked_and_reproducible(case):
    spec, e, om, pr = case
    phys = _points(spec, pr, 12, 23)
    ll0, g0, _ = _grad(e, phys)
    ll1, g1, _ = _grad(e, phys)
    assert np.array_equal(g0, g1) and np.array_equal(ll0, ll1)
    e.set_gradient_memory(3 * 100 * 33976 * 50 + (64 << 20))  # a few evaluations per chunk
    try:
        ll2, g2, _ = _grad(e, phys)
    finally:
        e.set_gradient_memory(0)
    assert np.array_equal(ll0, ll2) and np.array_equal(g0, g2)


def test_transmission_gradient_storing_shapes_are_bit_identical(case):
    """The storing forward pass with two wavenumbers per thread group (the default and the
    paired launch shapes) and with one (launch shape 32) stores the same opacity terms, pair
    sums and ray data, so the gradients are equal bit for bit; and the level sinks summed
    from the stored terms streamed through shared memory (even N) equal those recomputed
    from the level table (a gradient memory budget too small to store the terms)."""
    spec, e, om, pr = case
    phys = _points(spec, pr, 10, 27)
    ll0, g0, ng0 = _grad(e, phys)
    try:
        for rt in (32, 192, 160):
            e.set_launch(rt, 0)
            ll1, g1, ng1 = _grad(e, phys)
            assert np.array_equal(ll0, ll1) and np.array_equal(g0, g1) and np.array_equal(ng0, ng1), rt
    finally:
        e.set_launch(0, 0)
    assert e.N % 2 == 0
    e.set_gradient_memory(int(2.4 * 100 * e.N * 50))  # ray data of two evaluations, no opacity terms
    try:
        ll2, g2, ng2 = _grad(e, phys)
    finally:
        e.set_gradient_memory(0)
    assert np.array_equal(ll0, ll2) and np.array_equal(g0, g2) and np.array_equal(ng0, ng2)


def test_transmission_gradient_neglect_and_precision(case):
    spec, e, om, pr = case
    phys = _points(spec, pr, 3, 24)
    names = [p.description for p in pr]
    phys[1, names.index("H2O")] = 0.6  # mixing ratios summing above 1: neglected
    phys[1, names.index("CO")] = 0.6
    ll, g, ng = _grad(e, phys)
    assert ng[1] and ll[1] == -1e30 and np.all(g[1] == 0.0)
    assert not ng[0] and np.any(g[0] != 0.0)
    e.set_precision(1)  # the transmission adjoint runs in the double-float mode only
    try:
        with pytest.raises(_lib.EngineError):
            _grad(e, phys)
    finally:
        e.set_precision(0)


@pytest.fixture(scope="module", params=[0, 1], ids=["constant_gravity", "variable_gravity"])
def odd_case(request):
    """The transmission edge-case set (60 levels, 16469 points: an odd count, so pass 2b
    reads single wavenumbers instead of pairs), fitted mean molecular weight, error
    inflation and a 3-knot temperature profile; constant gravity, and the variable gravity
    of Atmosphere::calcAltitudeVariableGravity (src/forward_model/atmosphere/atmosphere.cpp:311-334),
    whose altitude tangent carries d z_{l-1} and the planet radius into each layer."""
    c = goldenlib.Case(os.path.join(goldenlib.GOLDEN_DIR, "transmission_edges.npz"))
    text = c.config_text()
    assert "variable_gravity 1" in text
    if request.param == 0:
        text = text.replace("variable_gravity 1", "variable_gravity 0")
    obs = c.observations()
    e = Engine(text, obs)
    om = oracle.OracleModel(text, obs)
    assert e.N % 2 == 1
    yield c, e, om, ("variable_gravity" if request.param else "constant_gravity")
    om.close()
    e.close()


def test_transmission_gradient_odd_point_count(odd_case):
    """Odd N, with and without the stored opacity terms, against the FP64 oracle's
    Richardson differences (cut-off disabled)."""
    c, e, om, tag = odd_case
    phys = np.array(c.params[:3], dtype=np.float64)
    e.set_tau_cutoff(float("inf"))
    om.set_tau_cutoff(float("inf"))
    try:
        ll_s, g_s, ng = _grad(e, phys)                       # opacity terms stored
        per_eval_without_terms = 60 * e.N * 50                # ray data of one evaluation (60 levels)
        e.set_gradient_memory(int(2.4 * per_eval_without_terms))  # too small to store the terms
        try:
            ll_r, g_r, _ = _grad(e, phys)                    # opacity terms recomputed
        finally:
            e.set_gradient_memory(0)
        assert np.array_equal(ll_s, ll_r) and np.array_equal(g_s, g_r)
        worst = 0.0
        for i in range(len(phys)):
            assert not ng[i]
            x = phys[i]
            assert abs(ll_s[i] - om.loglike(x)) <= 1e-8 + 1e-12 * abs(ll_s[i])
            d1 = np.array([_fd(om.loglike, x, j, 1e-5) for j in range(len(x))])
            d2 = np.array([_fd(om.loglike, x, j, 5e-6) for j in range(len(x))])
            fd = (4 * d2 - d1) / 3
            sa, sf = x * g_s[i], x * fd
            scale = np.max(np.abs(sf))
            for j in range(len(x)):
                err = abs(sa[j] - sf[j])
                if j == 12:  # cloud-top pressure (held-fixed cloud layers): zero
                    assert g_s[i][j] == 0.0
                    continue
                tol = 1e-6 * abs(sf[j]) + 1e-8 * scale + 2e-10 * abs(ll_s[i]) / 1e-5
                assert err <= tol, (i, j, sa[j], sf[j], err, tol)
                worst = max(worst, err / max(abs(sf[j]), 1e-300))
        _record("odd_point_count_fd_worst_rel_err_" + tag, worst)
    finally:
        e.set_tau_cutoff(10.0)
        om.set_tau_cutoff(10.0)
