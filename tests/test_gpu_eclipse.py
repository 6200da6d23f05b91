"""Secondary-eclipse (occultation) model on the GPU against the FP64 oracle.

Workload: the batched emission atmosphere (80 levels, 6 line species, 11001
points at 1 cm^-1) as an eclipse model with each stellar spectrum model
(blackbody with fitted T_eff, a stellar file, a 4 x 2 x 3 stellar grid), the
batched emission observations (R=100 spectrum with an instrument profile, 40
bins, 8 filters); 32 live points per batch. Gates: eclipse depths within 1e-6
relative, log L within 1e-8 + 1e-12 |log L| (the parity gates of the golden
cases)."""

import os

import numpy as np
import pytest

import goldenlib
import oracle
from bear_gb300 import synthetic as syn
from bear_gb300.config import observation_arrays, render_config
from bear_gb300.retrieval import Engine

pytestmark = pytest.mark.gpu


def _case(star_kind):
    spec = syn.CONFIGS["emission_batched"]
    root = syn.write_tables(spec, goldenlib.TABLE_ROOT)
    axes = None
    folder = os.path.join(goldenlib.TABLE_ROOT, "star_eclipse_batched_" + star_kind) + "/"
    if star_kind == "file":
        wl, fl = syn.star_spectrum(5600.0, 4.3, -0.2)
        goldenlib.write_star("file", {"star_wl": wl, "star_flux": fl}, folder)
        params = [folder + "star.dat"]
    elif star_kind == "grid":
        axes, gwl, gsp = syn.star_grid([4000.0, 4600.0, 5300.0, 6000.0], [4.0, 4.5], [-0.5, 0.0, 0.5])
        goldenlib.write_star("grid", {"star_axis0": axes[0], "star_axis1": axes[1], "star_axis2": axes[2],
                                      "star_grid_wl": gwl, "star_grid_spectra": gsp}, folder)
        params = [folder]
    else:
        params = []
    mc = syn.eclipse_model_config(spec, star_kind, params)
    text = render_config(syn.global_config(spec, root, "secondary_eclipse"), mc)
    obs = syn.observations(spec, "emission")
    pr = syn.eclipse_priors(spec, star_kind, axes)
    truth = syn.cube_to_physical(pr, np.full((1, len(pr)), 0.5))[0]
    om0 = oracle.OracleModel(text, [observation_arrays(o) for o in obs])
    _, m, _ = om0.forward(truth)
    off, parts = 0, []
    for o in obs:
        parts.append(m[off:off + len(o.data)])
        off += len(o.data)
    syn.attach_data(obs, parts, "transmission", spec.seed)
    arrays = [observation_arrays(o) for o in obs]
    return text, arrays, pr, truth, axes


@pytest.mark.parametrize("star_kind", ["blackbody", "file", "grid"])
def test_eclipse_batch_against_oracle(star_kind):
    import torch
    text, arrays, pr, truth, axes = _case(star_kind)
    e = Engine(text, arrays)
    om = oracle.OracleModel(text, arrays)
    B = 32
    phys = syn.cube_to_physical(pr, np.random.default_rng(11).uniform(0.02, 0.98, (B, len(pr))))
    phys[0] = truth
    if star_kind == "grid":
        phys[1, 2:5] = [5300.0, 4.0, 0.5]     # on grid nodes
        phys[2, 2:5] = [3500.0, 5.0, -1.0]    # below / above every axis: clamped
        phys[3, 2:5] = [5999.0, 4.49, 0.49]   # just inside the last cell
    ll, ng = e.loglike_batch(torch.tensor(phys, device="cuda"))
    ll, ng = ll.cpu().numpy(), ng.cpu().numpy()
    for i in list(range(6)) + [B - 1]:
        ref = om.loglike(phys[i])
        spec_ref, obs_ref, neg_ref = om.forward(phys[i])
        assert bool(ng[i]) == neg_ref
        assert abs(ll[i] - ref) <= 1e-8 + 1e-12 * abs(ref), (i, ll[i], ref)
        spec, obs, neg = e.compute_model(phys[i])
        assert neg == neg_ref
        assert goldenlib.rel_err(obs, obs_ref) < 1e-6
        assert goldenlib.rel_err(spec, spec_ref) < 1e-6
        assert ll[i] == e.loglike(phys[i])
    e.close()


def test_eclipse_fp64_and_double_float_paths_agree():
    import torch
    text, arrays, pr, truth, _ = _case("blackbody")
    e = Engine(text, arrays)
    phys = syn.cube_to_physical(pr, np.random.default_rng(12).uniform(0.02, 0.98, (16, len(pr))))
    P = torch.tensor(phys, device="cuda")
    ll_df, _ = e.loglike_batch(P)
    e.set_precision(1)
    ll_64, _ = e.loglike_batch(P)
    d = (ll_df - ll_64).abs().cpu().numpy()
    assert np.all(d <= 1e-8 + 1e-12 * ll_64.abs().cpu().numpy()), d.max()
    e.close()


def _fd(om, x, j, rel):
    h = rel * abs(x[j])
    xp, xm = x.copy(), x.copy()
    xp[j] += h
    xm[j] -= h
    return (om.loglike(xp) - om.loglike(xm)) / (2 * h)


@pytest.mark.parametrize("star_kind", ["blackbody", "file", "grid"])
def test_eclipse_gradient_against_oracle_finite_differences(star_kind):
    """The emission adjoint seeded through the planet / star ratio, with d/d(R_p/R_s) and
    the stellar parameters from the likelihood adjoint, against Richardson-extrapolated
    central differences (relative steps 1e-5, 5e-6) of the FP64 oracle, in
    log-parameter units; grid points are strictly inside a cell."""
    import torch
    text, arrays, pr, truth, axes = _case(star_kind)
    e = Engine(text, arrays)
    om = oracle.OracleModel(text, arrays)
    phys = syn.cube_to_physical(pr, np.random.default_rng(13).uniform(0.1, 0.9, (2, len(pr))))
    phys[0] = truth
    if star_kind == "grid":
        phys[0, 2:5] = [4300.0, 4.2, -0.2]
    ll, g, ng = e.grad_batch(torch.tensor(phys, device="cuda"))
    ll, g = ll.cpu().numpy(), g.cpu().numpy()
    names = [p.description for p in pr]
    for i in range(len(phys)):
        x = phys[i]
        assert not ng[i]
        assert abs(ll[i] - om.loglike(x)) <= 1e-8 + 1e-12 * abs(ll[i])
        d1 = np.array([_fd(om, x, j, 1e-5) for j in range(len(x))])
        d2 = np.array([_fd(om, x, j, 5e-6) for j in range(len(x))])
        fd = (4 * d2 - d1) / 3
        sa, sf = x * g[i], x * fd
        scale = np.max(np.abs(sf))
        for j, nm in enumerate(names):
            err = abs(sa[j] - sf[j])
            tol = 1e-6 * abs(sf[j]) + 1e-8 * scale + 2e-10 * abs(ll[i]) / 1e-5
            assert err <= tol, (star_kind, i, nm, sa[j], sf[j], err, tol)
    e.close()
