"""H- continuum (bound-free + free-free) in the batched emission workload (80 levels,
6 line species, 11001 points at 1 cm^-1 from 0.8 um, H, H- and e- in the chemistry)
against the FP64 oracle, and the double-float path against the FP64 path. Models
with the H- continuum, and transmission models with a power-law / KH cloud, have no gradient
(BEAR_ERR_UNSUPPORTED)."""

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


def test_hminus_gradient_is_rejected(case):
    import torch
    e, om, truth, ns = case
    with pytest.raises(_lib.EngineError) as ei:
        e.grad_batch(torch.tensor(truth[None, :], device="cuda"))
    assert ei.value.code == 4


def test_transmission_non_grey_cloud_gradient_is_rejected():
    """The non-grey clouds have an adjoint for emission models (test_gpu_gradient_cloud.py);
    the transmission adjoint rejects them."""
    import torch
    c = [goldenlib.Case(p) for p in goldenlib.golden_cases() if p.endswith("transmission_kh_cloud.npz")][0]
    e = Engine(c.config_text(), c.observations())
    try:
        with pytest.raises(_lib.EngineError) as ei:
            e.grad_batch(torch.tensor(c.params[:1], device="cuda"))
        assert ei.value.code == 4
    finally:
        e.close()
