"""Host-side set-up of the joint model (no GPU): the emission and transmission
models, each carrying the other's observations with likelihood weight 0, sample
one spectral grid (the condition for sharing their device tables)."""

import numpy as np

import goldenlib
from bear_gb300 import synthetic as syn
from bear_gb300.config import observation_arrays, render_config
from bear_gb300.joint import joint_observation_sets
from bear_gb300.retrieval import Engine

SPEC = syn.scaled(syn.CONFIGS["joint_large"], name="joint_small", nu_step=1.0, nb_levels=60,
                  species=syn.LINE_SPECIES[:4],
                  table=syn.TableSpec(6, 1e-6, 100.0, 8, 100.0, 3500.0, -22.5, 1.75))


def test_joint_models_share_one_grid():
    root = syn.write_tables(SPEC, goldenlib.TABLE_ROOT)

    def part(kind):
        text = render_config(syn.global_config(SPEC, root, kind), syn.model_config(SPEC, kind))
        return text, [observation_arrays(o) for o in syn.observations(SPEC, kind)]

    te, oe = part("emission")
    tt, ot = part("transmission")
    em, tr = joint_observation_sets(oe, ot)
    assert all(np.all(o.weight == 0) for o in em[len(oe):]) and all(np.all(o.weight == 0) for o in tr[len(ot):])
    e = Engine(te, em, prepare_only=True)
    t = Engine(tt, tr, prepare_only=True)
    try:
        assert e.N == t.N and np.array_equal(e.wavenumbers, t.wavenumbers)
        assert e.M == t.M == sum(o.n for o in em) == 900
        alone = Engine(te, oe, prepare_only=True)
        assert alone.N < e.N  # the transmission observations add grid points
        alone.close()
    finally:
        e.close()
        t.close()
