"""The benchmark configurations that the other GPU tests do not reach, at
their stated sizes, against the FP64 oracle:

  * config 5: the 40 A sphere with the 4,000-atom chain and 60 Q atoms in 2
    states (18,013 atoms; the chain displaces about half of the sphere's
    water).  Exact pair and Q lists, LRF multipoles, forces and per-state
    energies; then 1,000 FP64-master MD steps (lists every 10 steps) with no
    SHAKE, list-capacity or fixed-point failure, and the same parity again at
    the coordinates of step 1,000.
  * config 1: the 18 A droplet for its stated 1,000 steps, engine (FP64
    master) and oracle each from the same start.  The first 100 steps follow
    the oracle closely; after that the two trajectories separate as any two
    MD trajectories do, so the later steps are compared as averages.
"""
from collections import Counter

import numpy as np
import pytest

from listcheck import expand, oracle_records

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-5
E_KEYS = ["pp_el", "pp_vdw", "pw_el", "pw_vdw", "ww_el", "ww_vdw", "lrf", "qx_el", "qx_vdw", "q_bond", "q_angle",
          "q_torsion", "q_improper", "p_bond", "p_angle", "p_torsion", "p_improper"]
EQ_KEYS = ["qq_el", "qq_vdw", "qp_el", "qp_vdw", "qw_el", "qw_vdw", "q_bond", "q_angle", "q_torsion", "q_improper"]


def _bad(eg, eo, keys, rel=1e-5, absolute=2e-3):
    return [(k, eg[k], eo[k]) for k in keys if abs(eg[k] - eo[k]) > max(rel * abs(eo[k]), absolute)]


@pytest.fixture(scope="module")
def cfg5(engine_lib):
    from qsource_gb300 import synth
    return synth.config(5)


def _parity(s, e, o):
    """Lists, Q lists, LRF, forces and energies of engine e and oracle o on
    the same coordinates (both have built their lists)."""
    from test_gpu_parity import q_lists_of_oracle
    ex = expand(s, e.group_pairs())
    for lst in ("pp", "pw", "ww"):
        assert Counter(ex[lst]) == Counter(oracle_records(o, lst)), lst
    qp, qw = e.q_lists(0)
    atoms, wat, nrec_p, nrec_w = q_lists_of_oracle(o, int(s.nat_solute), int(s.nqat))
    assert np.array_equal(qp, atoms) and np.array_equal(qw, wat)
    assert nrec_p == int(s.nqat) * len(qp)
    g, r = e.lrf(), o.get_lrf()
    assert np.allclose(g[:, :3], r[:, :3], rtol=0, atol=1e-12)
    for lo, hi in ((3, 4), (4, 7), (7, 16), (16, 43)):
        scale = np.abs(r[:, lo:hi]).max()
        assert np.abs(g[:, lo:hi] - r[:, lo:hi]).max() <= 1e-5 * scale, (lo, hi)
    d, E, EQ = e.pot_energy(0, terms=0x1F)
    do, Eo, EQo = o.pot_energy(0x1F)
    err = float(np.sqrt(np.sum((d - do) ** 2) / np.sum(do ** 2)))
    assert err <= FORCE_RTOL, err
    assert not _bad(E, Eo, E_KEYS)
    for q, qo in zip(EQ, EQo):
        assert not _bad(q, qo, EQ_KEYS, rel=1e-6)
    return err


def test_cfg5_parity_and_1000_steps(cfg5):
    from oracle.oracle import Oracle
    from qsource_gb300.engine import Engine
    s = cfg5
    assert s.natom > 18000 and int(s.nqat) == 60 and int(s.nat_solute) == 4000
    e = Engine(s)
    e.make_pair_lists()
    o = Oracle(s)
    o.make_pair_lists()
    err0 = _parity(s, e, o)
    rows = e.run(1000, ene_every=100)[0]       # raises on any device status (SHAKE, lists, range, NaN)
    assert len(rows) == 10
    for _, E, EQ in rows:
        assert np.isfinite(E["potential"]) and np.isfinite(E["kinetic"]) and E["kinetic"] > 0
    x, v = e.coords(0)
    e2 = Engine(s)
    e2.set_coords(0, x, v)
    e2.make_pair_lists()
    o.set_coords(x, v)
    o.make_pair_lists()
    err1 = _parity(s, e2, o)
    print(f"config 5: force rel RMS {err0:.2e} at the start, {err1:.2e} after 1000 steps")


def test_cfg1_1000_steps_against_oracle(engine_lib):
    from oracle.oracle import Oracle
    from qsource_gb300 import synth
    from qsource_gb300.engine import Engine
    s = synth.config(1)
    e = Engine(s)
    rows = e.run(1000, ene_every=10)[0]
    o = Oracle(s)
    o.temperature()
    rc, orows, _, _ = o.md_run(1000)
    assert rc == 0 and len(rows) == 100
    pot_g = np.array([r[1]["potential"] for r in rows])
    kin_g = np.array([r[1]["kinetic"] for r in rows])
    pot_o = np.array([orows[r[0]]["potential"] for r in rows])
    kin_o = np.array([orows[r[0]]["kinetic"] for r in rows])
    early = np.array([r[0] for r in rows]) <= 100
    dpot = np.abs(pot_g - pot_o) / np.maximum(1.0, np.abs(pot_o))
    dkin = np.abs(kin_g - kin_o) / kin_o
    print("config 1, 1000 steps: early max rel dev pot %.2e kin %.2e; late means pot %.1f vs %.1f, kin %.1f vs %.1f"
          % (dpot[early].max(), dkin[early].max(), pot_g[50:].mean(), pot_o[50:].mean(), kin_g[50:].mean(),
             kin_o[50:].mean()))
    assert dpot[early].max() < 1e-3 and dkin[early].max() < 1e-3
    # steps 500-1000: block means of separated trajectories of one droplet
    assert abs(pot_g[50:].mean() - pot_o[50:].mean()) < 0.02 * abs(pot_o[50:].mean())
    assert abs(kin_g[50:].mean() - kin_o[50:].mean()) < 0.03 * kin_o[50:].mean()
