"""Host-side checks of the synthetic systems (no GPU): the generator builds
every benchmark configuration through the same start-up code as the
reference's inputs, and the FP64 oracle runs a short MD on them."""
import numpy as np
import pytest


@pytest.mark.parametrize("cfg", [1, 2])
def test_synthetic_configs_build_and_run(cfg):
    from oracle.oracle import Oracle
    from qsource_gb300 import synth
    s = synth.config(cfg)
    d = s.desc()
    assert d.natom == s.natom and d.thermostat == 0 and d.integrator == 0
    assert d.any_atom_lists == (1 if cfg != 1 else 0)
    o = Oracle(s)
    o.temperature()
    rc, rows, _, _ = o.md_run(3)
    assert rc == 0 and all(np.isfinite(r["potential"]) for r in rows)


def test_lambda_batch_members_are_the_batch():
    from qsource_gb300 import synth
    b = synth.lambda_batch(nwindows=3, replicas=2)
    for i, s in enumerate(b):
        t = synth.lambda_batch_member(i, nwindows=3, replicas=2)
        assert s.natom == t.natom and np.array_equal(s.x, t.x) and np.array_equal(s.crg, t.crg)
