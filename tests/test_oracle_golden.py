"""The FP64 oracle against the reference's own golden step-0 energies.

Pins (tests/golden/golden.json, written by tests/golden/make_golden.py):
  * tests/basic_tests/SPH_leap-frog_berendsen_benchmark.en row 1 of the
    reference: QEL QVdW EL VdW QBND QANG QTOR QIMP BND ANG TOR IMP (lower ==
    upper bound, printed to 0.01 kcal/mol);
  * tests/basic_tests/PBC_leap-frog_berendsen_benchmark.en row 1: the same
    12 columns for the periodic box (prep_PBC inputs, q_atom 24, lrf 24);
  * tests/test2/eval_test.sh:67 and tests/test3/eval_test.sh:67: the step-0
    "Q-surr." el/vdW line.
Step 0 follows qdyn's start-up (src/qdyn.f90:126-132): maxwell, initial
shaking, stop_cm_translation, then (in a box) put_back_in_box,
make_pair_lists and pot_energy.
"""
import os

import pytest

from conftest import golden_system

# the reference tree (qusers/qsource), when present: QSOURCE_REFERENCE names it
REF = os.environ.get("QSOURCE_REFERENCE", "")


def step0(system):
    from oracle.oracle import Oracle
    o = Oracle(system)
    o.maxwell(system.Tmaxw, int(system.seed))
    assert o.initial_shaking() == 0
    o.stop_cm_translation()
    if getattr(system, "use_pbc", 0):
        o.put_back_in_box()
    o.make_pair_lists()
    d, E, EQ = o.pot_energy()
    return o, d, E, EQ


def columns(E, EQ):
    q = EQ[0]
    return {
        "QEL": q["qp_el"] + q["qw_el"], "QVdW": q["qp_vdw"] + q["qw_vdw"],
        "EL": E["pp_el"] + E["pw_el"] + E["ww_el"], "VdW": E["pp_vdw"] + E["pw_vdw"] + E["ww_vdw"],
        "QBND": q["q_bond"], "QANG": q["q_angle"], "QTOR": q["q_torsion"], "QIMP": q["q_improper"],
        "BND": E["p_bond"], "ANG": E["p_angle"], "TOR": E["p_torsion"], "IMP": E["p_improper"],
    }


@pytest.mark.parametrize("name", ["basic_sph", "basic_pbc", "test2", "test3"])
def test_step0_matches_reference_golden(name, golden):
    s = golden_system(name)
    _, _, E, EQ = step0(s)
    got = columns(E, EQ)
    for col, want in golden[name].items():
        # the reference prints these with f10.2; the pin is the printed value
        assert round(got[col], 2) == pytest.approx(want, abs=1e-9), (name, col, got[col], want)


def test_golden_fixture_matches_reference_inputs():
    """The committed fixture is the parse of the reference's own inputs."""
    if not REF or not os.path.isdir(REF):
        pytest.skip("reference tree not mounted")
    import numpy as np

    import sys
    from conftest import GOLDEN
    sys.path.insert(0, GOLDEN)
    from make_golden import systems
    from qsource_gb300.system import System
    for name, (top, fep, inp) in systems(REF):
        a = System.from_files(top, fep, inp)
        b = golden_system(name)
        for k in ("x", "crg", "iac", "cgpatom", "shake_i", "excl_pairs", "pairs14", "qcrg", "bnd", "tor"):
            assert np.array_equal(np.asarray(getattr(a, k)), np.asarray(getattr(b, k))), (name, k)


def test_oracle_newton_third_law():
    """Internal forces of the pair terms sum to zero (momentum conservation)."""
    import numpy as np
    s = golden_system("test3")
    o, d, E, EQ = step0(s)
    d, _, _ = o.pot_energy(terms=0x1 | 0x2 | 0x4 | 0x8)
    tot = d.reshape(-1, 3).sum(axis=0)
    # LRF is a one-sided field approximation; the rest must cancel
    d2, _, _ = o.pot_energy(terms=0x2 | 0x4 | 0x8)
    assert np.abs(d2.reshape(-1, 3).sum(axis=0)).max() < 1e-8
    assert np.isfinite(tot).all()


def test_oracle_shake_restores_constraints():
    import numpy as np
    from oracle.oracle import Oracle
    s = golden_system("test3")
    o = Oracle(s)
    x = s.x.copy()
    rng = np.random.default_rng(5)
    x2 = x + rng.normal(0, 0.01, size=x.shape)
    it = o.shake(x.copy(), x2)
    assert it > 0
    i, j, d2 = s.shake_i, s.shake_j, s.shake_dist2
    r2 = ((x2.reshape(-1, 3)[i] - x2.reshape(-1, 3)[j]) ** 2).sum(1)
    # A constraint marked converged is never revisited, so later corrections in
    # the same molecule can move it again (src/md.f90:17606-17628): most
    # constraints end inside the tolerance, not all.
    rel = np.abs(r2 - d2) / d2
    assert np.median(rel) < 1e-4 and np.mean(rel < 1e-4) > 0.5
