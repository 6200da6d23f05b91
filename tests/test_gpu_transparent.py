"""Nearly transparent emission columns against the FP64 oracle: every line species at
mixing ratios of 0 and 1e-30 .. 1e-14 and no collision-induced absorption, so the layer
optical depths are exactly 0 (layers the reference skips) or fall to 1e-25 .. 1e-9.
There exp(-delta) rounds to 1 or to a few ulp below it, and the reference's
q = (a - 1)/delta keeps only the rounding of a: the
engine's recurrence (carried as J = I - B with (a - 1) rounded where the reference
rounds it) must reproduce those results, in the double-float and in the FP64 path."""

import os

import numpy as np
import pytest

import goldenlib
import oracle
from bear_gb300.retrieval import Engine

pytestmark = pytest.mark.gpu

VMRS = [0.0, 1e-30, 1e-24, 1e-20, 1e-17, 1e-14]  # 0: every layer has tau == 0 exactly (skipped)


@pytest.fixture(scope="module")
def case():
    c = goldenlib.Case(os.path.join(goldenlib.GOLDEN_DIR, "emission_plain.npz"))
    text = "".join(line + "\n" for line in c.config_text().splitlines() if not line.startswith("opacity CIA"))
    obs = c.observations()
    e = Engine(text, obs)
    yield c, e, oracle.OracleModel(text, obs)
    e.close()


def _params(c, vmr):
    p = np.array(c.params[0], dtype=np.float64)
    p[3:7] = vmr  # the four line species (general parameters: log g, scaling, distance)
    return p


@pytest.mark.parametrize("precision", [0, 1])
def test_transparent_columns_against_oracle(case, precision):
    c, e, om = case
    e.set_precision(precision)
    try:
        for vmr in VMRS:
            p = _params(c, vmr)
            spec_ref, obs_ref, neg_ref = om.forward(p)
            spec, obs, neg = e.compute_model(p)
            assert neg == neg_ref
            assert goldenlib.rel_err(spec, spec_ref) < 1e-6, vmr
            assert goldenlib.rel_err(obs, obs_ref) < 1e-6, vmr
            ref = om.loglike(p)
            assert abs(e.loglike(p) - ref) <= 1e-8 + 1e-12 * abs(ref), (vmr, e.loglike(p), ref)
    finally:
        e.set_precision(0)


def test_transparent_batch_matches_plain(case):
    import torch
    c, e, _ = case
    P = np.stack([_params(c, v) for v in VMRS])
    ll, _ = e.loglike_batch(torch.tensor(P, device="cuda"))
    ll = ll.cpu().numpy()
    for i, p in enumerate(P):
        assert ll[i] == e.loglike(p)
