"""The oracle's arithmetic combination rule (ivdw_rule 2, the reference's
nonbon2_* routines, src/md.f90:11354-13068).

Parity unpinned by reference data: the reference ships no system that uses
the arithmetic rule, so there is no golden energy for it.  These tests pin the oracle's restatement two ways:
  * the synthetic LJ types converted to the arithmetic form (radius R* and
    sqrt(eps) per type, qsource_gb300.synth._arithmetic_params) reproduce every
    same-type LJ curve, so the water-water LJ energy (O-O pairs only) equals
    the geometric rule's to 1e-9 relative and the Coulomb terms are identical;
  * the solute-solute and solute-water LJ energies equal an independent numpy
    evaluation of eps_ij (R*_i + R*_j)^12 / r^12 - 2 eps_ij (R*_i + R*_j)^6 / r^6
    (eps_ij = b_i b_j) over the oracle's own pair lists, to 1e-10 relative.
"""
import numpy as np


def _energies(s):
    from oracle.oracle import Oracle
    o = Oracle(s)
    o.make_pair_lists()
    _, E, EQ = o.pot_energy(0x1F)
    return o, E, EQ


def test_arithmetic_rule_reproduces_same_type_lj():
    from qsource_gb300 import synth
    _, Eg, _ = _energies(synth.config(1))
    _, Ea, _ = _energies(synth.config(1, vdw_rule=2))
    assert abs(Ea["ww_vdw"] - Eg["ww_vdw"]) <= 1e-9 * abs(Eg["ww_vdw"])
    for k in ("ww_el", "pw_el", "pp_el", "lrf"):
        assert Ea[k] == Eg[k], k


def test_arithmetic_pair_energies_match_numpy():
    from qsource_gb300 import synth
    qa = synth.neutral_charges(np.random.default_rng(5), 4, 0.4)
    s = synth.synthetic(14.0, 60, 4, np.stack([qa, np.zeros(4)], 1), (0.5, 0.5), 77, vdw_rule=2)
    o, E, _ = _energies(s)
    x = np.asarray(s.x).reshape(-1, 3)
    av, bv, iac = np.asarray(s.avdw), np.asarray(s.bvdw), np.asarray(s.iac)

    def lj(rows):
        i, j, c = rows[:, 0], rows[:, 1], rows[:, 2] - 1
        a = (av[iac[i], c] + av[iac[j], c]) ** 6
        b = bv[iac[i], c] * bv[iac[j], c]
        r2 = np.sum((x[j] - x[i]) ** 2, axis=1)
        return float(np.sum(b * a * a / r2 ** 6 - 2.0 * b * a / r2 ** 3))

    pp, pw = o.get_list("pp"), o.get_list("pw")
    assert len(pp) > 100 and len(pw) > 100
    assert abs(lj(pp) - E["pp_vdw"]) <= 1e-10 * max(1.0, abs(E["pp_vdw"]))
    assert abs(lj(pw) - E["pw_vdw"]) <= 1e-10 * max(1.0, abs(E["pw_vdw"]))
