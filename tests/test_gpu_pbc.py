"""Periodic box on the GPU against the FP64 oracle, through the C-ABI.

System: the reference's own PBC test (tests/basic_tests/prep_PBC: the 46-atom
ligand in 4,072 waters, 12,262 atoms in a 49.633 A cubic box; eq1.inp with
q_atom 24, lrf 24, solvent put back in the box at every list update), after
qdyn's start-up (maxwell, initial shaking, stop_cm_translation,
put_back_in_box); every test runs with its switch-atom lists and again with
any-atom lists (the reference ships no any-atom box output: that form is
pinned by the oracle's restatement only).

Tolerances (as tests/test_gpu_parity.py):
  * pair-list sets: exact;
  * LRF multipoles: |d phi| <= 1e-5 * max|phi| per component family;
  * forces: relative RMS <= 1e-5; energies 1e-5 relative or 2e-3 kcal/mol;
  * the reference's printed step-0 columns (PBC_leap-frog_berendsen_benchmark.en
    row 1) to their 2 decimals;
  * MD: recorded potential and kinetic energies 1e-4 relative, coordinates
    1e-4 A after 30 steps (two list updates, each with put_back_in_box).
"""
import copy
from collections import Counter

import numpy as np
import pytest

from conftest import golden_system
from listcheck import expand, oracle_records

pytestmark = pytest.mark.gpu

E_KEYS = ["pp_el", "pp_vdw", "pw_el", "pw_vdw", "ww_el", "ww_vdw", "lrf", "qx_el", "qx_vdw", "q_bond",
          "q_angle", "q_torsion", "q_improper", "p_bond", "p_angle", "p_torsion", "p_improper", "rst_protein"]
EQ_KEYS = ["qq_el", "qq_vdw", "qp_el", "qp_vdw", "qw_el", "qw_vdw", "q_bond", "q_angle", "q_torsion", "q_improper"]


def _oracle(s):
    from oracle.oracle import Oracle
    return Oracle(s)


def _engine(s):
    from qsource_gb300.engine import Engine
    return Engine(s)


@pytest.fixture(scope="module", params=["ref-switch_atom", "ref-any_atom", "synth-switch_atom", "synth-any_atom"])
def box(engine_lib, request):
    """The reference's PBC system with its own switch-atom lists
    (iuse_switch_atom = 1) and the same system with any-atom lists
    (iuse_switch_atom = 0: nbpplis2_box_lrf / nbpwlis2_box_lrf, src/md.f90:7241,
    :8745; every group pair's periodic shift from its first atom pair inside
    the cut-off); then the seeded synthetic cube of tests/test_oracle_box_any.py
    (an 80-atom chain of which 72 atoms are outside the Q region, so the
    solute-solute and solute-water lists that the reference's system leaves
    empty are exercised) in both forms."""
    src, form = request.param.split("-")
    if src == "synth":
        from test_oracle_box_any import synthetic_box
        return synthetic_box(form == "any_atom")
    g = golden_system("basic_pbc")
    g.any_atom_lists = 1 if form == "any_atom" else 0
    o = _oracle(g)
    o.maxwell(g.Tmaxw, int(g.seed))
    assert o.initial_shaking() == 0
    o.stop_cm_translation()
    o.put_back_in_box()
    g.x, g.v = o.coords()
    g.rand_state = o.rand_state()
    g.reference_box = True
    return g


def _close(eg, eo, keys):
    return [(k, eg[k], eo[k]) for k in keys if abs(eg[k] - eo[k]) > max(1e-5 * abs(eo[k]), 2e-3)]


def _rel_rms(a, b):
    return float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b ** 2)))


def _images(s, seed=3, frac=0.3):
    """The same system with a seeded subset of its solvent molecules moved by
    a whole box length along random axes (another periodic image of each).
    Solute molecules stay: the reference's sequence restraint to the
    geometric centre (p_restrain :15488-15516) takes no minimum image."""
    t = copy.copy(s)
    x = np.array(s.x, dtype=np.float64).reshape(-1, 3)
    rng = np.random.default_rng(seed)
    starts = list(np.asarray(s.istart_mol)) + [s.natom]
    L = np.asarray(s.boxlength)
    for m in range(int(s.nsolute_mol), len(starts) - 1):
        if rng.random() < frac:
            ax = rng.integers(0, 3)
            x[starts[m]:starts[m + 1], ax] += L[ax] * (1 if rng.random() < 0.5 else -1)
    t.x = x.ravel()
    return t


def test_pbc_pair_lists_exact(box):
    e = _engine(box)
    e.make_pair_lists()
    o = _oracle(box)
    o.make_pair_lists()
    ex = expand(box, e.group_pairs())
    for lst in ("pp", "pw", "ww"):
        assert Counter(ex[lst]) == Counter(oracle_records(o, lst)), lst


def test_pbc_lrf_multipoles(box):
    e = _engine(box)
    e.make_pair_lists()
    o = _oracle(box)
    o.make_pair_lists()
    g, r = e.lrf(), o.get_lrf()
    assert np.allclose(g[:, :3], r[:, :3], rtol=0, atol=1e-12)
    for lo, hi in ((3, 4), (4, 7), (7, 16), (16, 43)):
        scale = np.abs(r[:, lo:hi]).max()
        err = np.abs(g[:, lo:hi] - r[:, lo:hi]).max()
        assert err <= 1e-5 * scale, (lo, err, scale)


def test_pbc_forces_energies_and_golden_columns(box, golden):
    e = _engine(box)
    e.make_pair_lists()
    d, E, EQ = e.pot_energy(0, terms=0x1F)
    o = _oracle(box)
    o.make_pair_lists()
    do, Eo, EQo = o.pot_energy(0x1F)
    assert _rel_rms(d, do) <= 1e-5
    assert not _close(E, Eo, E_KEYS)
    for q, qo in zip(EQ, EQo):
        assert not _close(q, qo, EQ_KEYS)
    if box.any_atom_lists or not getattr(box, "reference_box", False):
        return   # the reference's printed row: its own system and switch-atom lists
    q = EQ[0]
    got = {"QEL": q["qp_el"] + q["qw_el"], "QVdW": q["qp_vdw"] + q["qw_vdw"],
           "EL": E["pp_el"] + E["pw_el"] + E["ww_el"], "VdW": E["pp_vdw"] + E["pw_vdw"] + E["ww_vdw"],
           "QBND": q["q_bond"], "QANG": q["q_angle"], "QTOR": q["q_torsion"], "QIMP": q["q_improper"],
           "BND": E["p_bond"], "ANG": E["p_angle"], "TOR": E["p_torsion"], "IMP": E["p_improper"]}
    for col, want in golden["basic_pbc"].items():
        assert round(got[col], 2) == pytest.approx(want, abs=1e-9), (col, got[col], want)


def test_pbc_results_do_not_depend_on_the_image(box):
    """Molecules moved by whole box lengths give the same lists, forces and
    energies (minimum images everywhere), on the GPU and in the oracle."""
    t = _images(box)
    e0, e1 = _engine(box), _engine(t)
    e0.make_pair_lists(); e1.make_pair_lists()
    assert Counter(map(tuple, np.sort(e0.group_pairs(), axis=1).tolist())) == \
        Counter(map(tuple, np.sort(e1.group_pairs(), axis=1).tolist()))
    d0, E0, EQ0 = e0.pot_energy(0, terms=0x1F)
    d1, E1, EQ1 = e1.pot_energy(0, terms=0x1F)
    assert _rel_rms(d1, d0) <= 1e-5
    assert not _close(E1, E0, E_KEYS)
    o = _oracle(t)
    o.make_pair_lists()
    do, Eo, _ = o.pot_energy(0x1F)
    assert _rel_rms(d1, do) <= 1e-5
    assert not _close(E1, Eo, E_KEYS)


def test_pbc_q_lists_exact(box):
    """nbqplist_box / nbqwlist_box (src/md.f90:10327, :10554): partners
    within Rcq of the Q switching atom, minimum image, rebuilt at every
    list update; equal to the oracle's record sets."""
    from test_gpu_parity import q_lists_of_oracle
    e = _engine(box)
    e.make_pair_lists()
    o = _oracle(box)
    o.make_pair_lists()
    qp, qw = e.q_lists(0)
    atoms, wat, nrec_p, nrec_w = q_lists_of_oracle(o, int(box.nat_solute), int(box.nqat))
    assert np.array_equal(qp, atoms) and np.array_equal(qw, wat)
    assert nrec_w == 3 * int(box.nqat) * len(qw)
    assert 0 < len(qw) <= int(box.nwat)


@pytest.mark.parametrize("precision", ["mixed", "fp64", "fp64_unfused"])
@pytest.mark.parametrize("start", ["in_box", "images"])
def test_pbc_md_matches_oracle(box, precision, start):
    """30 leap-frog Berendsen steps (0.1 fs, lists every 25 steps, solvent put
    back in the box before each list update).  From "images" the first
    put_back_in_box moves a third of the molecules: the engine and the oracle
    must move the same ones."""
    from qsource_gb300.abi import PRECISION
    s = _images(box) if start == "images" else box
    e = _engine(s)
    e.set_precision(PRECISION[precision])
    rows = e.run(30, ene_every=5)[0]
    o = _oracle(s)
    o.temperature()
    rc, orows, _, _ = o.md_run(30)
    assert rc == 0 and len(rows) == 6
    for r in rows:
        k = r[0]
        for key in ("potential", "kinetic"):
            g_, w_ = r[1][key], orows[k][key]
            assert abs(g_ - w_) <= 1e-4 * max(1.0, abs(w_)), (k, key, g_, w_)
    x, _ = e.coords(0)
    xo, _ = o.coords()
    assert np.abs(x - xo).max() < 1e-4
