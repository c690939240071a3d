"""The other p_restrain restraints on the GPU against the oracle: atom
position, distance and angle restraints (states 0, 1 and 2) and the sphere's
wall restraints, in the drop-in FP64 evaluation, the FP32 step form and 20 MD
steps; distance and angle restraints across the periodic box.  Tolerances as
tests/test_gpu_parity.py."""
import numpy as np
import pytest

from conftest import golden_system
from test_restraints_host import with_restraints

pytestmark = pytest.mark.gpu

E_KEYS = ["rst_protein", "rst_total", "potential"]


def _close(a, b, keys, rel=1e-5, ab=2e-3):
    return [(k, a[k], b[k]) for k in keys if abs(a[k] - b[k]) > max(rel * abs(b[k]), ab)]


@pytest.mark.parametrize("step", [False, True])
def test_restraint_forces_and_energies(engine_lib, step):
    from oracle.oracle import Oracle
    from qsource_gb300 import synth
    from qsource_gb300.abi import QGPU_TERMS_STEP_PRECISION
    from qsource_gb300.engine import Engine
    s = with_restraints(synth.config(1, lambdas=(0.7, 0.3)))
    e = Engine(s)
    e.make_pair_lists()
    terms = 0x1F | (QGPU_TERMS_STEP_PRECISION if step else 0)
    d, E, EQ = e.pot_energy(0, terms=terms)
    o = Oracle(s)
    o.make_pair_lists()
    do, Eo, EQo = o.pot_energy(0x1F)
    assert float(np.sqrt(np.sum((d - do) ** 2) / np.sum(do ** 2))) <= 1e-5
    assert not _close(E, Eo, ["rst_protein", "rst_total"], ab=2e-2 if step else 2e-3)
    for q, qo in zip(EQ, EQo):
        assert abs(q["restraint"] - qo["restraint"]) <= max(1e-5 * abs(qo["restraint"]), 2e-3)
        assert abs(q["total"] - qo["total"]) <= max(1e-5 * abs(qo["total"]), 2e-2 if step else 2e-3)


def test_restraints_across_the_box(engine_lib):
    from oracle.oracle import Oracle
    from qsource_gb300.engine import Engine
    s = with_restraints(golden_system("basic_pbc"), pbc=True)
    # a distance restraint between atoms on opposite faces of the box
    x = np.asarray(s.x).reshape(-1, 3)
    far = int(np.argmax(np.linalg.norm(x - x[0], axis=1)))
    s.rstdis_i = np.vstack([s.rstdis_i, [[0, far, 0]]]).astype(np.int32)
    s.rstdis_p = np.vstack([s.rstdis_p, [[3.0, 4.0, 2.0]]])
    e = Engine(s)
    e.make_pair_lists()
    d, E, EQ = e.pot_energy(0, terms=0x1F)
    o = Oracle(s)
    o.make_pair_lists()
    do, Eo, EQo = o.pot_energy(0x1F)
    assert float(np.sqrt(np.sum((d - do) ** 2) / np.sum(do ** 2))) <= 1e-5
    assert not _close(E, Eo, ["rst_protein", "rst_total"])


@pytest.mark.parametrize("precision", ["mixed", "fp64", "fp64_unfused"])
def test_restrained_md_matches_oracle(engine_lib, precision):
    from oracle.oracle import Oracle
    from qsource_gb300 import synth
    from qsource_gb300.abi import PRECISION
    from qsource_gb300.engine import Engine
    s = with_restraints(synth.config(1, lambdas=(0.7, 0.3)))
    e = Engine(s)
    e.set_precision(PRECISION[precision])
    rows = e.run(20, ene_every=5)[0]
    o = Oracle(s)
    o.temperature()
    rc, orows, oq, _ = o.md_run(20)
    assert rc == 0 and len(rows) == 4
    for r in rows:
        k = r[0]
        for key in ("potential", "kinetic", "rst_total"):
            g_, w_ = r[1][key], orows[k][key]
            assert abs(g_ - w_) <= 1e-4 * max(1.0, abs(w_)), (k, key, g_, w_)
    x, _ = e.coords(0)
    xo, _ = o.coords()
    assert np.abs(x - xo).max() < 1e-4
