"""The oracle's any-atom lists in a periodic box (nbpplis2_box_lrf,
nbpwlis2_box_lrf, src/md.f90:7241-7439, :8745-8900) on a seeded synthetic
periodic cube (31 A, an 80-atom chain with 8 Q atoms in 922 waters; the
reference's own PBC system has no solute atom outside its Q region, so its
solute-solute and solute-water lists are empty).

Parity unpinned by reference data: the reference ships no any-atom box
output.  The restatement is pinned by properties instead:
  * a group pair whose switch atoms are within the cut-off has some atom pair
    within it, so the any-atom record sets contain the switch-atom ones;
  * moving solvent molecules by whole box lengths changes no list, force or
    energy (minimum images and the shift records are image-independent);
  * every pair's shift record is an atom pair of the two groups within the
    cut-off (minimum image)."""
from collections import Counter

import numpy as np

from listcheck import oracle_records


def synthetic_box(any_atom, seed=77):
    """The seeded synthetic periodic cube of these tests (also used by the
    GPU tests)."""
    from qsource_gb300 import synth
    qa = synth.neutral_charges(np.random.default_rng(1), 8, 0.4)
    return synth.synthetic(11.0, 80, 8, np.stack([qa, np.zeros(8)], 1), (0.5, 0.5), seed, any_atom=any_atom,
                           box=31.0)


def _box(any_atom):
    return synthetic_box(any_atom)


def _oracle_lists(g):
    from oracle.oracle import Oracle
    o = Oracle(g)
    o.make_pair_lists()
    return o, {k: Counter(oracle_records(o, k)) for k in ("pp", "pw", "ww")}


def test_any_atom_box_lists_contain_the_switch_atom_lists():
    g_any, g_sw = _box(True), _box(False)
    assert np.array_equal(g_any.x, g_sw.x)
    _, la = _oracle_lists(g_any)
    _, ls = _oracle_lists(g_sw)
    for k in ("pp", "pw"):
        assert not (ls[k] - la[k]), k          # switch-atom records are all there
        assert sum(la[k].values()) >= sum(ls[k].values())
    assert la["ww"] == ls["ww"]                  # water pairs take the O-O test in both forms


def test_any_atom_box_is_image_independent():
    from oracle.oracle import Oracle
    from test_gpu_pbc import _images
    g = _box(True)
    o0, l0 = _oracle_lists(g)
    t = _images(g)
    assert not np.array_equal(np.asarray(t.x), np.asarray(g.x))
    o1, l1 = _oracle_lists(t)
    assert l0 == l1
    d0, E0, _ = o0.pot_energy(0x1F)
    d1, E1, _ = o1.pot_energy(0x1F)
    assert np.sqrt(np.sum((d1 - d0) ** 2) / np.sum(d0 ** 2)) < 1e-10
    for k in ("pp_el", "pp_vdw", "pw_el", "pw_vdw", "ww_el", "ww_vdw", "lrf"):
        assert abs(E1[k] - E0[k]) <= 1e-8 * max(1.0, abs(E0[k])), k
    assert isinstance(o1, Oracle)


def test_any_atom_box_shift_records_are_inside_pairs():
    """The shift record of every solute-solute record is an atom pair of the
    same two charge groups whose minimum-image distance is within Rcpp."""
    from oracle.oracle import Oracle
    g = _box(True)
    o = Oracle(g)
    o.make_pair_lists()
    rec = o.get_list_shift("pp")
    assert len(rec) > 0
    x = np.asarray(g.x).reshape(-1, 3)
    L = np.asarray(g.boxlength)
    grp = np.empty(g.natom, np.int64)
    for k in range(len(g.cgp_first)):
        grp[np.asarray(g.cgpatom[g.cgp_first[k]:g.cgp_last[k] + 1])] = k
    for i, j, si, sj in rec.tolist():
        assert grp[si] == grp[i] and grp[sj] == grp[j]
        d = x[sj] - x[si]
        d = d - L * np.round(d / L)
        assert d @ d <= float(g.Rcpp) ** 2 * (1 + 1e-12)
