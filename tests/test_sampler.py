"""Batched nested-sampling driver on CPU tensors with analytic likelihoods."""

import math

import numpy as np
import pytest

from bear_gb300.sampler import BatchedNestedSampler


def _gauss(mu, sigma):
    import torch

    def f(x):
        z = (x - mu) / sigma
        return (-0.5 * (z * z).sum(dim=1) - x.shape[1] * math.log(sigma * math.sqrt(2 * math.pi))).to(torch.float64)
    return f


@pytest.mark.parametrize("ndim,replace", [(3, 20), (5, 1)])
def test_evidence_and_posterior_of_a_gaussian(ndim, replace):
    """L = N(0.5, 0.05^2 I) on the unit cube: Z = 1 (the cube holds 10 sigma)."""
    import torch
    s = BatchedNestedSampler(_gauss(0.5, 0.05), ndim, n_live=300, batch=256, replace=replace, dlogz=0.05,
                             device="cpu", seed=ndim)
    r = s.run()
    assert abs(r.log_z) < 4 * r.log_z_err + 0.05, (r.log_z, r.log_z_err)
    w = torch.exp(r.log_weights)
    assert abs(float(w.sum()) - 1.0) < 1e-9
    mean = (w[:, None] * r.samples).sum(dim=0)
    std = torch.sqrt((w[:, None] * (r.samples - mean) ** 2).sum(dim=0))
    assert torch.all((mean - 0.5).abs() < 0.01), mean
    assert torch.all((std - 0.05).abs() < 0.01), std
    # information of a Gaussian in a unit volume: d (log(1 / (sigma sqrt(2 pi))) - 1/2)
    h_exact = ndim * (math.log(1 / (0.05 * math.sqrt(2 * math.pi))) - 0.5)
    assert abs(r.information - h_exact) < 0.3, (r.information, h_exact)


def test_rejected_points_never_enter():
    """-1e30 (neglected models) below every threshold: a likelihood that neglects half the
    cube gives log Z of the other half."""
    import torch

    def f(x):
        l = torch.zeros(x.shape[0], dtype=torch.float64)
        l[x[:, 0] < 0.5] = -1e30
        return l
    r = BatchedNestedSampler(f, 2, n_live=200, batch=128, dlogz=0.05, device="cpu", seed=1).run()
    assert abs(r.log_z - math.log(0.5)) < 4 * r.log_z_err + 0.05
    w = torch.exp(r.log_weights)
    assert float((w * (r.samples[:, 0] < 0.5)).sum()) < 1e-20
