"""The allocation-free single-evaluation entry point, bear_loglike_noalloc.

It exists for callers that must not allocate device memory while a likelihood
is evaluated (inside a CUDA stream capture, under another framework's memory
pool, in a per-point sampler callback). Its work buffers live in a fixed device
array instead of the model's growable workspace. This file is collected last so
that a run stopping at the first failure has run every other test first; it
also passes on its own in a fresh process (the array's address is looked up on
the first call for a device).
"""

import ctypes as C

import pytest

import goldenlib
from bear_gb300 import _lib
from bear_gb300.retrieval import Engine

pytestmark = pytest.mark.gpu

CASES = ["emission_edges", "transmission_edges"]


def _noalloc(engine, params_t, ll_t, ng_t, stream):
    lib = _lib.load()
    return lib.bear_loglike_noalloc(engine._h, C.c_void_p(params_t.data_ptr()), engine.P,
                                    C.c_void_p(ll_t.data_ptr()), C.c_void_p(ng_t.data_ptr()),
                                    C.c_void_p(stream))


@pytest.mark.parametrize("name", CASES)
def test_noalloc_matches_plain_loglike(name):
    import torch

    case = goldenlib.Case(f"{goldenlib.GOLDEN_DIR}/{name}.npz")
    eng = Engine(case.config_text(), case.observations())
    stream = torch.cuda.current_stream().cuda_stream
    ll = torch.empty(1, dtype=torch.float64, device="cuda")
    ng = torch.empty(1, dtype=torch.uint8, device="cuda")
    # two calls in a row on the shared scratch array, then the neglected parameter set
    for i in (0, 1, len(case.params) - 1):
        p = torch.tensor(case.params[i], dtype=torch.float64, device="cuda")
        ll.fill_(0.0)
        rc = _noalloc(eng, p, ll, ng, stream)
        assert rc == 0, _lib.load().bear_last_error().decode()
        torch.cuda.synchronize()
        expected = eng.loglike(case.params[i])           # the existing entry point
        assert bool(ng.item()) == bool(case.arrays["ref_neglect"][i])
        assert abs(ll.item() - expected) <= 1e-8, (i, ll.item(), expected)
        assert abs(ll.item() - case.arrays["ref_loglike"][i]) <= 1e-8 + 1e-12 * abs(expected)
    eng.close()


def test_noalloc_rejects_models_beyond_its_scratch():
    import torch

    case = goldenlib.Case(f"{goldenlib.GOLDEN_DIR}/transmission_edges.npz")
    text = case.config_text().replace("nb_grid_points 60", "nb_grid_points 512")
    eng = Engine(text, case.observations())
    p = torch.tensor(case.params[0], dtype=torch.float64, device="cuda")
    ll = torch.empty(1, dtype=torch.float64, device="cuda")
    ng = torch.empty(1, dtype=torch.uint8, device="cuda")
    rc = _noalloc(eng, p, ll, ng, torch.cuda.current_stream().cuda_stream)
    assert rc == 6  # BEAR_ERR_SIZE
    msg = _lib.load().bear_last_error().decode()
    assert "limited to 2097152 bytes" in msg
    eng.close()
