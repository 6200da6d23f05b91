"""The allocation-free single-evaluation entry point, bear_loglike_noalloc.

It exists for host applications that cannot call cudaMalloc while a likelihood
is evaluated: their device memory belongs to another framework's pool or to a
fixed budget set at start-up, or they evaluate from a per-point sampler callback
that must not block in the allocator. Its work buffers live in a fixed device
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
    # two calls in a row on the shared scratch array, then the neglected parameter set;
    # all device buffers exist before the first call
    rows = (0, 1, len(case.params) - 1)
    params = [torch.tensor(case.params[i], dtype=torch.float64, device="cuda") for i in rows]
    got = []
    free_after_first = model_bytes_after_first = None
    for n, p in enumerate(params):
        ll.fill_(0.0)
        rc = _noalloc(eng, p, ll, ng, stream)
        assert rc == 0, _lib.load().bear_last_error().decode()
        torch.cuda.synchronize()
        got.append((ll.item(), bool(ng.item())))
        if n == 0:
            # the first call on a device may load the library's device code (which holds
            # the scratch array); every later call must leave device memory as it is
            free_after_first = torch.cuda.mem_get_info()[0]
            model_bytes_after_first = eng.device_bytes()
        else:
            assert torch.cuda.mem_get_info()[0] == free_after_first, "device memory changed across a call"
            assert eng.device_bytes() == model_bytes_after_first, "the model's workspace grew"
    for i, (value, neglect) in zip(rows, got):
        expected = eng.loglike(case.params[i])           # the existing entry point
        assert neglect == bool(case.arrays["ref_neglect"][i])
        assert abs(value - expected) <= 1e-8, (i, value, expected)
        assert abs(value - case.arrays["ref_loglike"][i]) <= 1e-8 + 1e-12 * abs(expected)
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
