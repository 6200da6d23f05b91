"""Every evaluation call runs on the model's device and leaves the caller's current
device as it found it. With two GPUs: a model on GPU 1 evaluated while GPU 0 is
current gives the log-likelihood of the same model on GPU 0; with one GPU, the
current device is unchanged across each kind of call."""

import os

import numpy as np
import pytest

import goldenlib
from bear_gb300.retrieval import BatchEvaluator, Engine


def _device_count():
    try:
        import torch
        return torch.cuda.device_count()
    except Exception:
        return 0

pytestmark = pytest.mark.gpu


def _case():
    return goldenlib.Case(os.path.join(goldenlib.GOLDEN_DIR, "emission_edges.npz"))


def test_calls_keep_the_current_device():
    import torch

    c = _case()
    torch.cuda.set_device(0)
    e = Engine(c.config_text(), c.observations(), device=0)
    P = torch.tensor(c.params[:2], dtype=torch.float64, device="cuda:0")
    e.loglike(c.params[0])
    e.loglike_batch(P)
    e.grad_batch(P)
    ev = BatchEvaluator(e, P)
    ev()
    torch.cuda.synchronize()
    assert torch.cuda.current_device() == 0
    ev.close()
    e.close()


@pytest.mark.skipif(_device_count() < 2, reason="needs two GPUs")
def test_model_on_another_device():
    import torch

    c = _case()
    e0 = Engine(c.config_text(), c.observations(), device=0)
    e1 = Engine(c.config_text(), c.observations(), device=1)
    torch.cuda.set_device(0)
    ref = np.array([e0.loglike(p) for p in c.params])
    got = np.array([e1.loglike(p) for p in c.params])   # GPU 0 is current
    assert torch.cuda.current_device() == 0
    assert np.array_equal(ref, got)
    P1 = torch.tensor(c.params, dtype=torch.float64, device="cuda:1")
    ll, _ = e1.loglike_batch(P1)
    torch.cuda.synchronize(1)
    assert torch.cuda.current_device() == 0
    assert np.allclose(ll.cpu().numpy(), ref, rtol=0, atol=1e-8 + 1e-12 * np.abs(ref).max())
    e0.close()
    e1.close()
