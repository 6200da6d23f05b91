"""Transit depth with A impact parameters per layer (``transmission_annuli A``, not in the
reference) on the GPU against the FP64 oracle's restatement of the same integral: every
spectral and binned point within 1e-6 relative and log L within 1e-8 + 1e-12 |log L|, in
the double-float and the FP64 paths, for a non-grey (KH) cloud case and a variable-gravity
grey-cloud case. A = 1 gives the default kernel's results bit for bit; the captured,
autotuned batch and every launch shape agree; the adjoint gradient matches the oracle's
differences."""

import os

import numpy as np
import pytest

import goldenlib
import oracle
from bear_gb300.retrieval import Engine

pytestmark = pytest.mark.gpu

ANNULI = 10


def _text(c, annuli):
    return c.config_text() + f"transmission_annuli {annuli}\n"


@pytest.fixture(scope="module", params=["transmission_kh_cloud", "transmission_edges"])
def case(request):
    c = goldenlib.Case(os.path.join(goldenlib.GOLDEN_DIR, request.param + ".npz"))
    obs = c.observations()
    e = Engine(_text(c, ANNULI), obs)
    yield c, e, oracle.OracleModel(_text(c, ANNULI), obs)
    e.close()


def test_annuli_against_oracle(case):
    c, e, om = case
    for p in c.params:
        spec_ref, obs_ref, neg_ref = om.forward(p)
        spec, obs, neg = e.compute_model(p)
        assert neg == neg_ref
        if neg:
            continue
        assert goldenlib.rel_err(spec, spec_ref) < 1e-6
        assert goldenlib.rel_err(obs, obs_ref) < 1e-6
        ref = om.loglike(p)
        assert abs(e.loglike(p) - ref) <= 1e-8 + 1e-12 * abs(ref), (e.loglike(p), ref)


def test_annuli_batch_and_fp64_path(case):
    import torch
    c, e, om = case
    P = torch.tensor(np.repeat(c.params, 4, axis=0), device="cuda")
    ll_df, ng = e.loglike_batch(P)
    e.set_precision(1)
    try:
        ll_64, _ = e.loglike_batch(P)
    finally:
        e.set_precision(0)
    ll_df, ll_64 = ll_df.cpu().numpy(), ll_64.cpu().numpy()
    for i in range(len(P)):
        if bool(ng[i]):
            continue
        ref = om.loglike(c.params[i // 4])
        assert abs(ll_df[i] - ref) <= 1e-8 + 1e-12 * abs(ref)
        assert abs(ll_64[i] - ref) <= 1e-8 + 1e-12 * abs(ref)
        assert ll_df[i] == ll_df[(i // 4) * 4]


def test_one_annulus_is_the_default_kernel(case):
    c, _, _ = case
    obs = c.observations()
    e1 = Engine(_text(c, 1), obs)
    e0 = Engine(c.config_text(), obs)
    try:
        for p in c.params:
            s1, o1, _ = e1.compute_model(p)
            s0, o0, _ = e0.compute_model(p)
            assert np.array_equal(s1, s0) and np.array_equal(o1, o0)
    finally:
        e1.close()
        e0.close()


def _fd(f, x, j, rel):
    h = rel * abs(x[j])
    xp, xm = x.copy(), x.copy()
    xp[j] += h
    xm[j] -= h
    return (f(xp) - f(xm)) / (2 * h)


def test_annuli_gradient_against_oracle(case):
    """The adjoint with A rays per layer (tr_adjoint_pass2a_annuli: the first, partial
    segments' interpolated extinction, the impact radii between the levels, the finer
    trapezoid) against the oracle's Richardson differences of the same integral, with the
    tau > 10 cut-off disabled in both; the cloud-top pressure places whole layers (zero
    gradient). KH cloud case: the golden set's last two points (at the first, the cloud
    bottom moves by a level within the difference step); edge case: its first three."""
    import torch
    c, e, om = case
    if c.name == "transmission_kh_cloud":
        phys = np.array(c.params[1:], dtype=np.float64)
        top = phys.shape[1] - 1
    else:
        phys = np.array(c.params[:3], dtype=np.float64)
        top = 12
    e.set_tau_cutoff(float("inf"))
    om.set_tau_cutoff(float("inf"))
    try:
        ll, g, ng = e.grad_batch(torch.tensor(phys, device="cuda"))
        ll, g, ng = ll.cpu().numpy(), g.cpu().numpy(), ng.cpu().numpy()
        ll_f, _ = e.loglike_batch(torch.tensor(phys, device="cuda"))
        for i in range(len(phys)):
            assert not ng[i]
            x = phys[i]
            assert abs(ll[i] - om.loglike(x)) <= 1e-8 + 1e-12 * abs(ll[i])
            assert abs(ll[i] - float(ll_f[i])) <= 1e-9 + 1e-13 * abs(ll[i])
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
                assert err <= tol, (c.name, i, j, sa[j], sf[j], err, tol)
    finally:
        e.set_tau_cutoff(10.0)
        om.set_tau_cutoff(10.0)


def test_annuli_gradient_with_cutoff(case):
    """With the tau > 10 cut-off (held fixed by the adjoint): a finite gradient, log L equal
    to the batched forward pass's within rounding (the storing pass runs 4 threads per
    wavenumber), and d/dR_s (every depth scales as 1 / R_s^2, no cut-off moves) against
    Richardson differences of the engine."""
    import torch
    c, e, _ = case
    phys = np.array(c.params, dtype=np.float64)
    ll, g, ng = e.grad_batch(torch.tensor(phys, device="cuda"))
    ll, g, ng = ll.cpu().numpy(), g.cpu().numpy(), ng.cpu().numpy()
    ll2, ng2 = e.loglike_batch(torch.tensor(phys, device="cuda"))
    ll2 = ll2.cpu().numpy()
    js = 2  # R_s
    f = lambda p: float(e.loglike_batch(torch.tensor(p[None, :], device="cuda"))[0][0])
    for i in range(len(phys)):
        assert bool(ng[i]) == bool(ng2[i])
        if ng[i]:
            continue
        assert np.all(np.isfinite(g[i]))
        assert abs(ll[i] - ll2[i]) <= 1e-9 + 1e-13 * abs(ll[i])
        x = phys[i]
        fd = (4 * _fd(f, x, js, 5e-6) - _fd(f, x, js, 1e-5)) / 3
        assert abs(g[i][js] - fd) <= 1e-7 * abs(fd), (i, g[i][js], fd)


def test_annuli_autotuned_graph_and_shapes(case):
    """The captured, autotuned batch equals the uncaptured batch, and every launch shape
    (threads per wavenumber x rays per group) gives log L within rounding of the default."""
    import torch
    from bear_gb300.retrieval import BatchEvaluator
    c, e, om = case
    P = torch.tensor(np.repeat(c.params, 3, axis=0), device="cuda")
    ll_ref, ng_ref = e.loglike_batch(P)
    ll_ref = ll_ref.cpu().numpy()
    ev = BatchEvaluator(e, P)
    try:
        ll_g, ng_g = ev()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(ng_g.cpu().numpy(), ng_ref.cpu().numpy())
        shape_ll = {}
        for rt in (16, 32, 64):
            e.set_launch(rt, 0)
            shape_ll[rt] = e.loglike_batch(P)[0].cpu().numpy()
        e.set_launch(0, 0)
        assert np.array_equal(ll_g.cpu().numpy(), shape_ll[ev.rt_threads if ev.rt_threads in shape_ll else 32])
        for rt, ll in shape_ll.items():
            ok = ~ng_ref.cpu().numpy().astype(bool)
            assert np.all(np.abs(ll[ok] - ll_ref[ok]) <= 1e-9 + 1e-13 * np.abs(ll_ref[ok])), rt
    finally:
        ev.close()
