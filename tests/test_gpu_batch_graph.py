"""Captured batches (CUDA graph) and the launch-shape autotuner.

The graph replays the batched kernel sequence; its log-likelihoods must equal
the stream-launched batched path bit for bit, for the parameters it was
captured with and for new parameters written into its buffer. The autotuner
may pick any launch shape, and every shape computes each wavenumber with the
same code, so results are unchanged bit for bit."""

import numpy as np
import pytest

import goldenlib
import oracle
from bear_gb300 import _lib
from bear_gb300 import synthetic as syn
from bear_gb300.config import observation_arrays, render_config
from bear_gb300.retrieval import BatchEvaluator, Engine

pytestmark = pytest.mark.gpu


def _engine(name, kind):
    spec = syn.CONFIGS[name]
    root = syn.write_tables(spec, goldenlib.TABLE_ROOT)
    text = render_config(syn.global_config(spec, root, kind), syn.model_config(spec, kind))
    obs = syn.observations(spec, kind)
    om = oracle.OracleModel(text, [observation_arrays(o) for o in obs])
    _, m, _ = om.forward(syn.truth_parameters(spec, kind))
    off, parts = 0, []
    for o in obs:
        parts.append(m[off:off + len(o.data)])
        off += len(o.data)
    syn.attach_data(obs, parts, kind, spec.seed)
    return spec, Engine(text, [observation_arrays(o) for o in obs])


def _live(spec, kind, n, seed):
    import torch
    pr = syn.priors(spec, kind)
    cube = np.random.default_rng(seed).uniform(size=(n, len(pr)))
    return torch.tensor(syn.cube_to_physical(pr, cube), device="cuda")


@pytest.mark.parametrize("name,kind", [("emission_batched", "emission"), ("transmission_plain", "transmission")])
def test_graph_replay_equals_batched_path(name, kind):
    import torch
    spec, e = _engine(name, kind)
    try:
        P0 = _live(spec, kind, 48, 1)
        ref0, ng0 = e.loglike_batch(P0)
        ev = BatchEvaluator(e, P0, autotune=True)
        assert ev.rt_threads in ((16, 32, 64, 160, 176, 192, 208, 224) if kind == "transmission" else (64, 128, 256))
        ll, ng = ev()
        torch.cuda.synchronize()
        assert torch.equal(ll, ref0) and torch.equal(ng, ng0)
        P1 = _live(spec, kind, 48, 2)
        ll, ng = ev(P1)
        torch.cuda.synchronize()
        ref1, ng1 = e.loglike_batch(P1)  # after the autotune: same results as any launch shape
        assert torch.equal(ll, ref1) and torch.equal(ng, ng1)
        e.set_launch(0, 0)
        ref1b, _ = e.loglike_batch(P1)
        assert torch.equal(ref1b, ref1)
        ev.close()
    finally:
        e.close()


def test_graph_refuses_replay_after_reallocation():
    spec, e = _engine("emission_batched", "emission")
    try:
        P = _live(spec, "emission", 8, 3)
        ev = BatchEvaluator(e, P, autotune=False)
        ev()
        e.loglike_batch(_live(spec, "emission", 16, 4))  # grows the work buffers
        with pytest.raises(_lib.EngineError):
            ev()
    finally:
        e.close()  # destroys the evaluator's graph first


def test_transmission_launch_shapes_are_bit_identical():
    """Every transmission launch shape, one wavenumber or two per thread group, gives the
    same transit depths and log-likelihoods bit for bit (batched and single-evaluation
    paths); the batch's last block is partly past the grid in the wider shapes."""
    import torch
    spec, e = _engine("transmission_plain", "transmission")
    try:
        P = _live(spec, "transmission", 24, 5)
        p3 = P[3].cpu().numpy()
        ref = None
        for rt in (32, 16, 64, 160, 176, 192, 208, 224, 0):
            e.set_launch(rt, 0)
            ll, ng = e.loglike_batch(P)
            sp, binned, _ = e.compute_model(p3)
            torch.cuda.synchronize()
            if ref is None:
                ref = (ll.clone(), ng.clone(), sp.copy(), binned.copy())
                continue
            assert torch.equal(ll, ref[0]) and torch.equal(ng, ref[1]), rt
            assert np.array_equal(sp, ref[2]) and np.array_equal(binned, ref[3]), rt
    finally:
        e.set_launch(0, 0)
        e.close()
