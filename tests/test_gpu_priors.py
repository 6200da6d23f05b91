"""Prior transform on the device (bear_model_set_priors / bear_prior_transform_batch /
bear_loglike_cube_batch / bear_batch_graph_create_cube) against the host mirror of
the reference's transforms, on the batched-emission workload (512 live points)."""

import numpy as np
import pytest

import goldenlib
import oracle
from bear_gb300 import synthetic as syn
from bear_gb300.config import Prior, observation_arrays, render_config
from bear_gb300.retrieval import Engine, Priors

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    spec = syn.CONFIGS["emission_batched"]
    root = syn.write_tables(spec, goldenlib.TABLE_ROOT)
    text = render_config(syn.global_config(spec, root, "emission"), syn.model_config(spec, "emission"))
    obs = syn.observations(spec, "emission")
    om0 = oracle.OracleModel(text, [observation_arrays(o) for o in obs])
    _, m, _ = om0.forward(syn.truth_parameters(spec, "emission"))
    off, parts = 0, []
    for o in obs:
        parts.append(m[off:off + len(o.data)])
        off += len(o.data)
    syn.attach_data(obs, parts, "emission", spec.seed)
    e = Engine(text, [observation_arrays(o) for o in obs])
    pr = syn.priors(spec, "emission")
    # exercise every prior type: a Gaussian distance, a linked T ratio
    pr[2] = Prior("gaussian", "distance", [10.0, 0.3], "pc")
    names = [p.description for p in pr]
    pr[names.index("T ratio 5")] = Prior("linked", "T ratio 5", [names.index("T ratio 4") + 1])
    yield e, pr
    e.close()


def test_device_transform_matches_host(case):
    import torch
    e, pr = case
    e.set_priors(pr)
    cube = np.random.default_rng(5).uniform(size=(512, e.P))
    cube[0] = 0.0
    cube[1] = 1.0
    dev = e.prior_transform_batch(torch.tensor(cube, device="cuda")).cpu().numpy()
    host = Priors(pr).cube_to_physical_batch(cube)
    finite = np.isfinite(host)
    assert np.array_equal(np.isfinite(dev), finite)
    assert np.array_equal(dev[~finite], host[~finite])  # erfinv(+-1) = +-inf on both sides
    err = np.abs(dev[finite] - host[finite]) / np.maximum(np.abs(host[finite]), 1e-300)
    # one rounding of the log-uniform exponent x (the device contracts a + u (b - a) into
    # an FMA) moves 10^x by ln(10) |x| 2^-53 relative: ~2e-15 at x = -8
    assert err.max() < 1e-14, err.max()


def test_cube_batch_equals_transform_then_batch(case):
    import torch
    e, pr = case
    e.set_priors(pr)
    cube = torch.tensor(np.random.default_rng(6).uniform(0.01, 0.99, size=(256, e.P)), device="cuda")
    ll, ng, par = e.loglike_cube_batch(cube)
    par2 = e.prior_transform_batch(cube)
    ll2, ng2 = e.loglike_batch(par2)
    assert torch.equal(par, par2) and torch.equal(ll, ll2) and torch.equal(ng, ng2)


def test_captured_cube_graph(case):
    import ctypes as C
    import torch
    from bear_gb300 import _lib
    e, pr = case
    e.set_priors(pr)
    B = 128
    cube = torch.tensor(np.random.default_rng(7).uniform(0.01, 0.99, size=(B, e.P)), device="cuda")
    par = torch.empty_like(cube)
    ll = torch.empty(B, dtype=torch.float64, device="cuda")
    ng = torch.empty(B, dtype=torch.uint8, device="cuda")
    g = C.c_void_p()
    lib = _lib.load()
    _lib.check(lib.bear_batch_graph_create_cube(e._h, C.c_void_p(cube.data_ptr()), B, e.P, C.c_void_p(par.data_ptr()),
                                                C.c_void_p(ll.data_ptr()), C.c_void_p(ng.data_ptr()), C.byref(g)))
    try:
        for seed in (8, 9):
            cube.copy_(torch.tensor(np.random.default_rng(seed).uniform(0.01, 0.99, size=(B, e.P))))
            _lib.check(lib.bear_batch_graph_launch(g, C.c_void_p(torch.cuda.current_stream().cuda_stream)))
            ref_ll, ref_ng, ref_par = e.loglike_cube_batch(cube)
            torch.cuda.synchronize()
            assert torch.equal(ll, ref_ll) and torch.equal(par, ref_par)
    finally:
        lib.bear_batch_graph_destroy(g)


def test_prior_errors(case):
    from bear_gb300 import _lib
    e, pr = case
    with pytest.raises(_lib.EngineError):
        e.set_priors(pr[:-1])                       # wrong count
    bad = list(pr)
    bad[3] = Prior("linked", "x", [len(pr) + 5])
    with pytest.raises(_lib.EngineError):
        e.set_priors(bad)                           # link out of range


def test_device_transform_matches_the_reference_binary():
    """bear_prior_transform_batch against Retrieval::convertCubeParameters of the reference
    binary (tests/golden/priors.npz): uniform, log-uniform, delta and linked priors with
    every unit, on the emission edge-case model (12 parameters), 64 hypercube points."""
    import json
    import os

    import torch

    z = np.load(os.path.join(goldenlib.GOLDEN_DIR, "priors.npz"))
    meta = json.loads(bytes(z["meta"]).decode())
    base = goldenlib.Case(os.path.join(goldenlib.GOLDEN_DIR, meta["base_case"] + ".npz"))
    e = Engine(base.config_text(), base.observations())
    try:
        e.set_priors([Prior(t, d, p, u) for t, d, p, u in meta["priors"]])
        dev = e.prior_transform_batch(torch.tensor(z["cube"], device="cuda")).cpu().numpy()
    finally:
        e.close()
    ref = z["ref_physical"]
    err = np.abs(dev - ref) / np.maximum(np.abs(ref), 1e-300)
    # the log-uniform exponent a + u (b - a) is one FMA on the device: one rounding of it
    # moves 10^x by ln(10) |x| 2^-53 relative (~2e-15 at x = -9)
    assert err.max() < 1e-14, err.max()
