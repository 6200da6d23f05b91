"""The batched nested-sampling driver on the engine: live points, proposals, prior
transform and likelihood all on the device (Engine.loglike_cube_batch). Case: the
blackbody secondary-eclipse golden case with the data-generating parameter set as
the truth; R_p/R_s and T0 free (uniform), everything else fixed by delta priors."""

import numpy as np
import pytest

import goldenlib
from bear_gb300.config import Prior
from bear_gb300.retrieval import Engine
from bear_gb300.sampler import BatchedNestedSampler

pytestmark = pytest.mark.gpu


def test_nested_sampling_recovers_the_truth():
    import torch
    c = [goldenlib.Case(p) for p in goldenlib.golden_cases() if p.endswith("eclipse_blackbody.npz")][0]
    e = Engine(c.config_text(), c.observations())
    truth = c.params[0]
    # R_p/R_s and T0 of [log g, R_p/R_s, T_eff, 3 species, T0, 5 T ratios, shift]
    free = {1: (0.06, 0.16), 6: (1000.0, 3000.0)}
    pr = [Prior("uniform", f"p{j}", list(free[j])) if j in free else Prior("delta", f"p{j}", [float(v)])
          for j, v in enumerate(truth)]
    e.set_priors(pr)

    def loglike(cube):
        ll, _, _ = e.loglike_cube_batch(cube)
        return ll

    r = BatchedNestedSampler(loglike, e.P, n_live=120, batch=2048, dlogz=0.1, device="cuda", seed=3).run()
    w = torch.exp(r.log_weights)
    phys = e.prior_transform_batch(r.samples.contiguous())
    assert abs(float(w.sum()) - 1.0) < 1e-9
    assert r.n_calls > 0 and np.isfinite(r.log_z)
    for j in free:
        mean = float((w * phys[:, j]).sum())
        std = float(torch.sqrt((w * (phys[:, j] - mean) ** 2).sum()))
        assert abs(mean - truth[j]) < 5 * std + 1e-12 * abs(truth[j]), (j, mean, std, truth[j])
        assert std < 0.2 * (free[j][1] - free[j][0])  # the data constrain both
    e.close()
