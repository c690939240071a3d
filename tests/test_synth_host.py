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


def test_descriptor_outlives_later_descriptors():
    """A descriptor keeps its arrays alive when later descriptors of the same
    system are made (an engine built after an oracle of the same system must
    not free the oracle's arrays): every pointer of the first descriptor is
    still the address of an array that it holds after more descriptors and a
    collection, and the oracle built on it gives the same energies."""
    import ctypes as C
    import gc

    from oracle.oracle import Oracle
    from qsource_gb300 import synth
    from qsource_gb300.abi import SystemDesc
    s = synth.config(1)
    o = Oracle(s)
    o.make_pair_lists()
    d0, E0, _ = o.pot_energy()
    for _ in range(3):
        s.desc()
    gc.collect()
    held = {a.ctypes.data for a in o._desc._keep}
    for name, typ in SystemDesc._fields_:
        if typ is C.c_void_p and getattr(o._desc, name):
            assert getattr(o._desc, name) in held, name
    o.make_pair_lists()
    d1, E1, _ = o.pot_energy()
    assert np.array_equal(d0, d1) and E0 == E1
