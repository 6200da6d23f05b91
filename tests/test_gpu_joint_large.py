"""The large joint workload at its full size, against the FP64 oracle.

Emission + transmission models sharing one spectral grid and one set of device
tables: 150 levels, 12 line species + 2 CIA tables on 15 log-p x 30 T nodes,
1000-26000 cm^-1 at 0.25 cm^-1 (96307 model points once the four observations'
ranges are applied), four observations with 900 bins and Gaussian instrument
profiles of resolving power 100-3000, a batch of 1024 parameter sets.

At this size the level table holds 63000 rows x 96307 points (6.1e9 entries, past
2^31), the batch's spectra 9.9e7 values, and the gradient runs in chunks whose
stored intensities reach ~2e9 values. Rows spread over the whole batch (first,
middle, last) are compared with the oracle: the batched log L (both the plain
batched call and the captured graph), and through the single-evaluation path the
high-resolution spectrum and the binned spectra of each model. The gradient of the
full batch is computed with two different chunkings (the emission adjoint's stored
intensities for all 1024 evaluations would need 236 GB, so B = 1024 always runs in
chunks) and checked bit for bit, and for two rows against central differences of
the oracle (tangent-ray cut-off disabled in both, where log L is smooth).

Reference paths: src/forward_model/transmission/transmission_spectrum.cpp:32-154,
src/radiative_transfer/short_characteristics.cpp:39-125,
src/spectral_grid/spectral_band_convolve.cpp:44-144, src/retrieval/retrieval.cpp:314-369.
"""

import json
import os

import numpy as np
import pytest

import goldenlib
import oracle
from bear_gb300 import synthetic as syn
from bear_gb300.config import observation_arrays, render_config
from bear_gb300.joint import JointBatchEvaluator, JointEngine, joint_observation_sets

pytestmark = pytest.mark.gpu

SPEC = syn.CONFIGS["joint_large"]
B = SPEC.batch                  # 1024
ROWS = (0, 1, B // 2, B - 1)    # compared with the oracle
REPORT = {}


def _record(key, value):
    REPORT[key] = value
    out = os.environ.get("BEAR_JOINT_LARGE_REPORT")
    if out:
        with open(out, "w") as f:
            json.dump(REPORT, f, indent=1)


def _part(kind, root):
    """Config text and observations of one model, data = the oracle's model at the
    seeded truth plus noise."""
    text = render_config(syn.global_config(SPEC, root, kind), syn.model_config(SPEC, kind))
    obs = syn.observations(SPEC, kind)
    om = oracle.OracleModel(text, [observation_arrays(o) for o in obs])
    _, m, _ = om.forward(syn.truth_parameters(SPEC, kind))
    om.close()
    off, parts = 0, []
    for o in obs:
        parts.append(m[off:off + len(o.data)])
        off += len(o.data)
    syn.attach_data(obs, parts, kind, SPEC.seed)
    return text, [observation_arrays(o) for o in obs]


@pytest.fixture(scope="module")
def large():
    oracle.set_threads(os.cpu_count() or 1)
    root = syn.write_tables(SPEC, goldenlib.TABLE_ROOT)
    te, oe = _part("emission", root)
    tt, ot = _part("transmission", root)
    j = JointEngine(te, oe, tt, ot)
    em_sets, tr_sets = joint_observation_sets(oe, ot)
    ome, omt = oracle.OracleModel(te, em_sets), oracle.OracleModel(tt, tr_sets)
    assert j.N == ome.N == omt.N == 96307
    yield j, ome, omt
    ome.close()
    omt.close()
    j.close()


def _batch(j):
    """B live points drawn over both models' priors (seeded), the truth in row 0."""
    rng = np.random.default_rng(SPEC.seed + 4242)
    out = []
    for kind in ("emission", "transmission"):
        pr = syn.priors(SPEC, kind)
        phys = syn.cube_to_physical(pr, rng.uniform(0.05, 0.95, (B, len(pr))))
        phys[0] = syn.truth_parameters(SPEC, kind)
        out.append(phys)
    p = np.concatenate(out, axis=1)
    assert p.shape[1] == j.P
    return p


def test_joint_large_forward_against_oracle(large):
    import torch

    j, ome, omt = large
    phys = _batch(j)
    P = torch.tensor(phys, device="cuda")
    ll, ng = j.loglike_batch(P)
    ev = JointBatchEvaluator(j, P)
    ll_g, ng_g = ev()
    torch.cuda.synchronize()
    assert torch.equal(ll, ll_g) and torch.equal(ng, ng_g)
    ev.close()
    ll, ng = ll.cpu().numpy(), ng.cpu().numpy()
    worst = {"loglike_abs": 0.0, "loglike_rel": 0.0, "spectrum_rel": 0.0, "binned_rel": 0.0}
    for i in ROWS:
        pe, pt = phys[i, :j.Pe], phys[i, j.Pe:]
        ref_e, ref_t = ome.loglike(pe), omt.loglike(pt)
        assert not ng[i]
        ref = ref_e + ref_t
        err = abs(ll[i] - ref)
        assert err <= 2e-8 + 1e-12 * (abs(ref_e) + abs(ref_t)), (i, ll[i], ref)
        worst["loglike_abs"] = max(worst["loglike_abs"], err)
        worst["loglike_rel"] = max(worst["loglike_rel"], err / abs(ref))
        for eng, om, p in ((j.emission, ome, pe), (j.transmission, omt, pt)):
            spec, binned, neg = eng.compute_model(p)
            o_spec, o_bin, o_neg = om.forward(p)
            assert neg == o_neg
            es, eb = goldenlib.rel_err(spec, o_spec), goldenlib.rel_err(binned, o_bin)
            assert es <= 1e-6 and eb <= 1e-6, (i, es, eb)
            worst["spectrum_rel"] = max(worst["spectrum_rel"], es)
            worst["binned_rel"] = max(worst["binned_rel"], eb)
    _record("forward_worst", worst)


def _fd(f, x, j, rel):
    h = rel * abs(x[j])
    xp, xm = x.copy(), x.copy()
    xp[j] += h
    xm[j] -= h
    return (f(xp) - f(xm)) / (2 * h)


def test_joint_large_gradient_chunked_and_against_oracle(large):
    import torch

    j, ome, omt = large
    phys = _batch(j)
    P = torch.tensor(phys, device="cuda")
    j.transmission.set_tau_cutoff(float("inf"))
    omt.set_tau_cutoff(float("inf"))
    try:
        ll_a, g_a, ng_a = j.grad_batch(P)                        # default memory budget (32 GiB)
        for eng in (j.emission, j.transmission):
            eng.set_gradient_memory(6 << 30)                      # smaller chunks
        try:
            ll_b, g_b, ng_b = j.grad_batch(P)
        finally:
            for eng in (j.emission, j.transmission):
                eng.set_gradient_memory(0)
        torch.cuda.synchronize()
        assert torch.equal(ll_a, ll_b) and torch.equal(g_a, g_b) and torch.equal(ng_a, ng_b)
        ll, g = ll_a.cpu().numpy(), g_a.cpu().numpy()
        assert np.all(np.isfinite(g))
        names_e = [p.description for p in syn.priors(SPEC, "emission")]
        names_t = [p.description for p in syn.priors(SPEC, "transmission")]
        # emission: log g, an abundance, the bottom temperature; transmission: an abundance,
        # the bottom temperature (R_p and R_s are fixed by delta priors but differentiable)
        checks = [("emission", names_e.index("log g")), ("emission", names_e.index("CH4")),
                  ("emission", names_e.index("T0")), ("transmission", names_t.index("H2O")),
                  ("transmission", names_t.index("T0")), ("transmission", names_t.index("R_s"))]
        worst = 0.0
        for i in (0, B - 1):
            pe, pt = phys[i, :j.Pe], phys[i, j.Pe:]
            for kind, jj in checks:
                om, x, off = (ome, pe, 0) if kind == "emission" else (omt, pt, j.Pe)
                fd = (4 * _fd(om.loglike, x, jj, 5e-6) - _fd(om.loglike, x, jj, 1e-5)) / 3
                ad = g[i, off + jj]
                err = abs(ad - fd) * abs(x[jj])
                scale = abs(fd * x[jj])
                tol = 1e-6 * scale + 2e-10 * abs(ll[i]) / 1e-5
                assert err <= tol, (i, kind, jj, ad, fd, err, tol)
                worst = max(worst, err / max(scale, 1e-300))
        _record("gradient_fd_worst_rel", worst)
    finally:
        j.transmission.set_tau_cutoff(10.0)
        omt.set_tau_cutoff(10.0)
