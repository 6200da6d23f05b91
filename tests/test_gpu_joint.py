"""Joint emission + transmission likelihood on one spectral grid with shared tables.

A reduced copy of the large joint workload (60 levels, 4 line species + 2 CIA,
1000-26000 cm^-1 at 1 cm^-1, the same four observations with resolving powers
100-3000): the two models must sample one grid, the second model must reuse the
first model's device tables, and each half of the joint log-likelihood must match
the FP64 oracle built with the same observation sets (each model carrying the
other's observations with likelihood weight 0)."""

import numpy as np
import pytest

import goldenlib
import oracle
from bear_gb300 import synthetic as syn
from bear_gb300.config import observation_arrays, render_config
from bear_gb300.joint import JointBatchEvaluator, JointEngine, joint_observation_sets

pytestmark = pytest.mark.gpu

SPEC = syn.scaled(syn.CONFIGS["joint_large"], name="joint_small", nu_step=1.0, nb_levels=60,
                  species=syn.LINE_SPECIES[:4],
                  table=syn.TableSpec(6, 1e-6, 100.0, 8, 100.0, 3500.0, -22.5, 1.75))


def _part(kind, root):
    text = render_config(syn.global_config(SPEC, root, kind), syn.model_config(SPEC, kind))
    obs = syn.observations(SPEC, kind)
    om = oracle.OracleModel(text, [observation_arrays(o) for o in obs])
    _, m, _ = om.forward(syn.truth_parameters(SPEC, kind))
    off, parts = 0, []
    for o in obs:
        parts.append(m[off:off + len(o.data)])
        off += len(o.data)
    syn.attach_data(obs, parts, kind, SPEC.seed)
    return text, [observation_arrays(o) for o in obs]


@pytest.fixture(scope="module")
def joint():
    root = syn.write_tables(SPEC, goldenlib.TABLE_ROOT)
    te, oe = _part("emission", root)
    tt, ot = _part("transmission", root)
    j = JointEngine(te, oe, tt, ot)
    em_sets, tr_sets = joint_observation_sets(oe, ot)
    yield j, oracle.OracleModel(te, em_sets), oracle.OracleModel(tt, tr_sets)
    j.close()


def _points(n, seed):
    rng = np.random.default_rng(seed)
    pe = syn.cube_to_physical(syn.priors(SPEC, "emission"), rng.uniform(0.05, 0.95, (n, len(syn.priors(SPEC, "emission")))))
    pt = syn.cube_to_physical(syn.priors(SPEC, "transmission"),
                              rng.uniform(0.05, 0.95, (n, len(syn.priors(SPEC, "transmission")))))
    pe[0] = syn.truth_parameters(SPEC, "emission")
    pt[0] = syn.truth_parameters(SPEC, "transmission")
    return np.concatenate([pe, pt], axis=1)


def test_one_grid_and_shared_tables(joint):
    j, ome, omt = joint
    assert j.emission.N == j.transmission.N == ome.N == omt.N
    assert np.array_equal(j.emission.wavenumbers, j.transmission.wavenumbers)
    shared, nbytes = j.transmission.table_sharing()
    assert shared and nbytes > 0
    assert not j.emission.table_sharing()[0]


def test_joint_loglike_against_oracle(joint):
    import torch
    j, ome, omt = joint
    phys = _points(12, 1)
    ll, ng = j.loglike_batch(torch.tensor(phys, device="cuda"))
    ll = ll.cpu().numpy()
    for i in (0, 1, 2, 11):
        pe, pt = phys[i, :j.Pe], phys[i, j.Pe:]
        ref_e, ref_t = ome.loglike(pe), omt.loglike(pt)
        if ng[i]:
            assert ll[i] == -1e30
            continue
        ref = ref_e + ref_t
        tol = 2e-8 + 1e-12 * (abs(ref_e) + abs(ref_t))
        assert abs(ll[i] - ref) <= tol, (i, ll[i], ref)


def test_joint_graph_and_neglect(joint):
    import torch
    j, ome, omt = joint
    phys = _points(16, 2)
    P = torch.tensor(phys, device="cuda")
    ref, ng_ref = j.loglike_batch(P)
    ev = JointBatchEvaluator(j, P)
    ll, ng = ev()
    torch.cuda.synchronize()
    assert torch.equal(ll, ref) and torch.equal(ng, ng_ref)
    # a transmission temperature below the 50 K clamp neglects the joint row
    ti = j.Pe + [p.description for p in syn.priors(SPEC, "transmission")].index("T0")
    phys[3, ti] = 20.0
    ll, ng = ev(torch.tensor(phys, device="cuda"))
    torch.cuda.synchronize()
    assert bool(ng[3]) and ll[3].item() == -1e30
    ev.close()
