"""GPU engine vs the FP64 oracle on identical inputs, through the C-ABI.

Tolerances (pair terms run in FP32 with hi/lo coordinate differences, sums in
FP64 / int64 fixed point):
  * pair-list sets: exact (same (i, j, LJcod) records as the reference loops);
  * forces: relative RMS  sqrt(sum|dF|^2 / sum|F|^2) <= 1e-5;
  * energies: |dE| <= 1e-5 * (sum of |terms| scale) -- see ENERGY_TOL below;
  * LRF multipoles: |d phi| <= 1e-5 * max|phi| per component family;
  * SHAKE (drop-in, FP64): 1e-9 absolute on coordinates;
  * MD (the FP64-master step, and the mixed form with its float master
    state and FP32 SHAKE): recorded potential and kinetic energies 1e-4
    relative, coordinates 1e-4 A after 20 steps;
  * bit-identity where the arithmetic is the same: batch vs single
    trajectory, one vs several graph branches, run to run.
"""
from collections import Counter

import numpy as np
import pytest

from conftest import golden_system
from listcheck import expand, oracle_records

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-5
ENERGY_REL = 1e-5       # relative to |E| ...
ENERGY_ABS = 2e-3       # ... or absolute kcal/mol for terms that nearly cancel
STEP_PAIR_ENERGY_ABS = 0.05   # FP32 pair-energy sums, see test_step_precision_forces


def _engine(systems):
    from qsource_gb300.engine import Engine
    return Engine(systems)


def _oracle(s):
    from oracle.oracle import Oracle
    return Oracle(s)


@pytest.fixture(scope="module")
def systems(engine_lib):
    from qsource_gb300 import synth
    # cfg2/cfg4 use the any-atom cut-off (nb*lis2*); cfg2sw is cfg2 with the
    # switch-atom cut-off, which the reference's own golden systems also use
    out = {"cfg1": synth.config(1), "cfg2": synth.config(2), "cfg4": synth.config(4),
           "cfg2sw": synth.config(2, any_atom=False)}
    # the arithmetic combination rule (ivdw_rule 2) and per-state Q atom types
    out["cfg1ar"] = synth.config(1, vdw_rule=2)
    out["cfg1qv"] = synth.config(1, qvdw=True)
    out["cfg1arqv"] = synth.config(1, vdw_rule=2, qvdw=True)
    out["cfg2ar"] = synth.config(2, vdw_rule=2)
    # arithmetic rule with LJ on the water hydrogens (nonbon2_ww / nonbon2_qw
    # take LJ on every water atom)
    out["cfg1arh"] = synth.config(1, vdw_rule=2, water_h_lj=True)
    out["cfg1arqvh"] = synth.config(1, vdw_rule=2, qvdw=True, water_h_lj=True)
    g = golden_system("basic_sph")
    o = _oracle(g)
    o.maxwell(g.Tmaxw, int(g.seed))
    assert o.initial_shaking() == 0
    o.stop_cm_translation()
    g.x, g.v = o.coords()
    g.rand_state = o.rand_state()   # the random stream continues after maxwell
    out["golden"] = g
    return out


def rel_rms(a, b):
    return float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b ** 2)))


def energies_close(eg, eo, keys):
    bad = []
    for k in keys:
        if abs(eg[k] - eo[k]) > max(ENERGY_REL * abs(eo[k]), ENERGY_ABS):
            bad.append((k, eg[k], eo[k]))
    return bad


E_KEYS = ["pp_el", "pp_vdw", "pw_el", "pw_vdw", "ww_el", "ww_vdw", "lrf", "qx_el", "qx_vdw", "q_bond",
          "q_angle", "q_torsion", "q_improper", "p_bond", "p_angle", "p_torsion", "p_improper", "rst_shell",
          "rst_solvent_radial", "rst_protein", "rst_water_pol"]
EQ_KEYS = ["qq_el", "qq_vdw", "qp_el", "qp_vdw", "qw_el", "qw_vdw", "q_bond", "q_angle", "q_torsion", "q_improper"]


@pytest.mark.parametrize("name", ["golden", "cfg1", "cfg2", "cfg2sw", "cfg4"])
def test_pair_lists_exact(systems, name):
    s = systems[name]
    e = _engine(s)
    e.make_pair_lists()
    o = _oracle(s)
    o.make_pair_lists()
    ex = expand(s, e.group_pairs())
    for lst in ("pp", "pw", "ww"):
        assert Counter(ex[lst]) == Counter(oracle_records(o, lst)), lst


@pytest.mark.parametrize("name", ["golden", "cfg1", "cfg2", "cfg2sw"])
def test_lrf_multipoles(systems, name):
    s = systems[name]
    e = _engine(s)
    e.make_pair_lists()
    o = _oracle(s)
    o.make_pair_lists()
    g, r = e.lrf(), o.get_lrf()
    assert np.allclose(g[:, :3], r[:, :3], rtol=0, atol=1e-12)
    for lo, hi in ((3, 4), (4, 7), (7, 16), (16, 43)):
        scale = np.abs(r[:, lo:hi]).max()
        err = np.abs(g[:, lo:hi] - r[:, lo:hi]).max()
        assert err <= 1e-5 * scale, (lo, err, scale)


@pytest.mark.parametrize("name", ["golden", "cfg1", "cfg2", "cfg2sw", "cfg4", "cfg1ar", "cfg1qv", "cfg1arqv", "cfg2ar",
                                  "cfg1arh", "cfg1arqvh"])
def test_forces_and_energies(systems, name):
    s = systems[name]
    e = _engine(s)
    e.make_pair_lists()
    d, E, EQ = e.pot_energy(0, terms=0x1F)
    o = _oracle(s)
    o.make_pair_lists()
    do, Eo, EQo = o.pot_energy(0x1F)
    assert rel_rms(d, do) <= FORCE_RTOL
    assert not energies_close(E, Eo, E_KEYS)
    for q, qo in zip(EQ, EQo):
        assert not energies_close(q, qo, EQ_KEYS)


def _ragged_check(batch, qfree=()):
    """Step-0 forces and energies of every trajectory of the batch against the
    oracle (per-state Q energies zero for the trajectories in qfree), then 20
    FP64-master MD steps against the oracle's dynamics of each."""
    from qsource_gb300.abi import PRECISION
    e = _engine(batch)
    e.make_pair_lists()
    for t, s in enumerate(batch):
        d, E, EQ = e.pot_energy(t, terms=0x1F)
        o = _oracle(s)
        o.make_pair_lists()
        do, Eo, EQo = o.pot_energy(0x1F)
        assert rel_rms(d, do) <= FORCE_RTOL
        assert not energies_close(E, Eo, E_KEYS)
        for q, qo in zip(EQ, EQo):
            assert not energies_close(q, qo, EQ_KEYS)
        if t in qfree:
            assert len(EQ) == 1 and all(EQ[0][k] == 0.0 for k in ("qq_el", "qp_el", "qw_el", "qp_vdw", "qw_vdw"))
    e = _engine(batch)
    e.set_precision(PRECISION["fp64"])
    rows = e.run(20, ene_every=10)
    for t, s in enumerate(batch):
        o = _oracle(s)
        o.temperature()
        rc, orows, oq, T = o.md_run(20)
        assert rc == 0 and len(rows[t]) == 2
        for r in rows[t]:
            k = r[0]
            assert abs(r[1]["potential"] - orows[k]["potential"]) <= 1e-4 * max(1.0, abs(orows[k]["potential"]))
        x, _ = e.coords(t)
        xo, _ = o.coords()
        assert np.abs(x - xo).max() < 1e-4


def test_ragged_batch_with_a_trajectory_without_q_atoms(systems):
    """A batch of uneven content: a 9 A droplet around a 20-atom chain with no
    Q atoms and one state (a plain MD system), beside the two-state Q droplet."""
    from qsource_gb300 import synth
    plain = synth.synthetic(9.0, 20, 0, np.zeros((0, 1)), (1.0,), 5)
    _ragged_check([plain, systems["cfg1"]], qfree=(0,))


def test_ragged_batch_with_a_water_only_trajectory(systems):
    """A droplet of water alone (no solute, no Q atoms: no solute items, no
    solute groups in the lists, no bonded terms) beside the two-state Q
    droplet."""
    from qsource_gb300 import synth
    water = synth.synthetic(9.0, 0, 0, np.zeros((0, 1)), (1.0,), 5)
    assert water.nat_solute == 0 and water.nbonds_solute == 0
    _ragged_check([systems["cfg1"], water], qfree=(1,))


def test_golden_columns_on_gpu(systems, golden):
    """The GPU path reproduces the reference's printed step-0 values."""
    s = systems["golden"]
    e = _engine(s)
    e.make_pair_lists()
    _, E, EQ = e.pot_energy(0)
    q = EQ[0]
    got = {"QEL": q["qp_el"] + q["qw_el"], "QVdW": q["qp_vdw"] + q["qw_vdw"],
           "EL": E["pp_el"] + E["pw_el"] + E["ww_el"], "VdW": E["pp_vdw"] + E["pw_vdw"] + E["ww_vdw"],
           "QBND": q["q_bond"], "QANG": q["q_angle"], "QTOR": q["q_torsion"], "QIMP": q["q_improper"],
           "BND": E["p_bond"], "ANG": E["p_angle"], "TOR": E["p_torsion"], "IMP": E["p_improper"]}
    for col, want in golden["basic_sph"].items():
        assert round(got[col], 2) == pytest.approx(want, abs=1e-9), (col, got[col], want)


def test_shake_matches_oracle(systems):
    s = systems["cfg1"]
    e = _engine(s)
    o = _oracle(s)
    rng = np.random.default_rng(1)
    xx = s.x.copy()
    x = xx + rng.normal(0, 0.005, size=xx.shape)
    xg, _ = e.shake(0, xx, x)
    xo = x.copy()
    assert o.shake(xx.copy(), xo) >= 1
    assert np.abs(xg - xo).max() < 1e-9


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name,ene_every", [("cfg1", 1), ("cfg1", 5), ("cfg1arqv", 5), ("cfg2ar", 5), ("cfg1arqvh", 5)])
def test_short_md_matches_oracle(systems, name, ene_every, precision):
    """20 Berendsen leap-frog steps with SHAKE and lists every 10 steps, with
    the FP64 master (FP64 x, v, leap-frog and SHAKE; FP32 pair terms) and the
    mixed form (float master state, FP32 SHAKE and bonded terms on unrecorded
    steps); recorded steps evaluate energies in FP64."""
    from qsource_gb300.abi import PRECISION
    s = systems[name]
    e = _engine(s)
    e.set_precision(PRECISION[precision])
    rows = e.run(20, ene_every=ene_every)[0]
    o = _oracle(s)
    o.temperature()
    rc, orows, oq, T = o.md_run(20)
    assert rc == 0 and len(rows) == 20 // ene_every
    for r in rows:
        k = r[0]
        pg, po = r[1]["potential"], orows[k]["potential"]
        assert abs(pg - po) <= 1e-4 * max(1.0, abs(po)), (k, pg, po)
        kg, ko = r[1]["kinetic"], orows[k]["kinetic"]
        assert abs(kg - ko) <= 1e-4 * ko, (k, kg, ko)
    x, _ = e.coords(0)
    xo, _ = o.coords()
    assert np.abs(x - xo).max() < 1e-4


@pytest.mark.parametrize("name", ["cfg1", "cfg2ar"])
def test_fused_fp64_step_equals_unfused(systems, name):
    """The fused FP64-master update (leap-frog, SHAKE of one water per lane
    and the step's end in one kernel) against the separate FP64 update,
    SHAKE and step-end kernels over 30 steps (three list updates): the same
    arithmetic up to the association of products, with temperatures from the
    same exact integer sums, so coordinates agree to 1e-10 A, velocities to
    1e-9 and recorded energies to 1e-9 relative."""
    from qsource_gb300.abi import PRECISION
    s = systems[name]
    out = []
    for p in ("fp64", "fp64_unfused"):
        e = _engine(s)
        e.set_precision(PRECISION[p])
        rows = e.run(30, ene_every=5)[0]
        x, v = e.coords(0)
        out.append((rows, x, v))
    (ra, xa, va), (rb, xb, vb) = out
    assert len(ra) == len(rb) == 6
    assert np.abs(xa - xb).max() < 1e-10
    assert np.abs(va - vb).max() < 1e-9
    for a, b in zip(ra, rb):
        for key in ("potential", "kinetic"):
            assert abs(a[1][key] - b[1][key]) <= 1e-9 * max(1.0, abs(b[1][key])), (a[0], key)


def test_fp64_step_float_coordinates_are_the_rounded_master(systems):
    """The FP64-master step forms the pair kernels' float coordinates
    (hi = float(x - origin), lo = float(x - origin - hi), and the packed
    water records) from the bits of x with integer instructions.  Forming
    them again from the same x with the conversion instructions
    (qgpu_set_coords) must give bit-identical step-precision forces and
    energies."""
    from qsource_gb300.abi import PRECISION, QGPU_TERMS_STEP_PRECISION
    s = systems["cfg2ar"]
    e = _engine(s)
    e.set_precision(PRECISION["fp64"])
    e.run(15, ene_every=0)
    d1, E1, EQ1 = e.pot_energy(0, terms=0x1F | QGPU_TERMS_STEP_PRECISION)
    x, v = e.coords(0)
    e.set_coords(0, x, v)
    d2, E2, EQ2 = e.pot_energy(0, terms=0x1F | QGPU_TERMS_STEP_PRECISION)
    assert np.array_equal(d1, d2)
    assert E1 == E2


@pytest.mark.parametrize("precision", ["mixed", "fp64", "fp64_unfused"])
@pytest.mark.parametrize("integrator", [0, 1])
@pytest.mark.parametrize("thermostat", [0, 1, 2])
def test_thermostats_match_oracle(systems, thermostat, integrator, precision):
    """The reference's sphere test system (water polarisation, sequence,
    shell and radial restraints; 0.1 fs steps) for 20 steps with each
    thermostat (Berendsen, Langevin with the reference's random stream,
    Nose-Hoover chain) and integrator (leap-frog, velocity-verlet), against
    the FP64 oracle from the same start: recorded potential and kinetic
    energies to 1e-4 relative, coordinates to 1e-4 A."""
    import copy
    from qsource_gb300.abi import PRECISION
    s = copy.copy(systems["golden"])
    s.thermostat, s.integrator = thermostat, integrator
    e = _engine(s)
    e.set_precision(PRECISION[precision])
    rows = e.run(20, ene_every=5)[0]
    o = _oracle(s)
    o.temperature()
    rc, orows, _, _ = o.md_run(20)
    assert rc == 0 and len(rows) == 4
    for r in rows:
        k = r[0]
        for key in ("potential", "kinetic"):
            g_, w_ = r[1][key], orows[k][key]
            assert abs(g_ - w_) <= 1e-4 * max(1.0, abs(w_)), (k, key, g_, w_)
    x, _ = e.coords(0)
    xo, _ = o.coords()
    assert abs(x - xo).max() < 1e-4


def q_lists_of_oracle(o, nsol, nq):
    """Partner atoms of the oracle's nbqp records and O atoms of its nbqw
    records, with the record counts."""
    qp, qw = o.get_list("qp"), o.get_list("qw")
    atoms = np.unique(qp[:, 1]) if len(qp) else np.zeros(0, np.int32)
    wat = qw[:, 1] - (qw[:, 1] - nsol) % 3 if len(qw) else np.zeros(0, np.int32)
    return atoms, np.unique(wat), len(qp), len(qw)


@pytest.mark.parametrize("rcq", [None, 12.0])
@pytest.mark.parametrize("name", ["golden", "cfg1", "cfg2", "cfg2sw", "cfg4"])
def test_q_lists_exact(systems, name, rcq):
    """The Q-atom lists (nbqplist / nbqplis2, nbqwlist; src/md.f90:10215,
    :9946, :10464) are index work: the engine's solute partners and waters
    equal the oracle's record sets exactly, every partner paired with every
    Q atom (3 records per water and Q atom), skipped atoms (:10288) absent.
    With Rcq = 12 A the lists are rebuilt at every list update and cut
    through the system; they are compared again after 20 MD steps."""
    import copy
    s = copy.copy(systems[name])
    if rcq:
        s.Rcq = rcq
    nsol, nq = int(s.nat_solute), int(s.nqat)
    e = _engine(s)
    e.make_pair_lists()
    o = _oracle(s)
    o.make_pair_lists()
    for stage in ("start", "after 20 steps"):
        qp, qw = e.q_lists(0)
        atoms, wat, nrec_p, nrec_w = q_lists_of_oracle(o, nsol, nq)
        assert np.array_equal(qp, atoms), stage
        assert np.array_equal(qw, wat), stage
        assert nrec_p == nq * len(qp) and nrec_w == 3 * nq * len(qw), stage
        if rcq:
            assert 0 < len(qw) < int(s.nwat), stage
        if stage == "start":
            if not rcq:
                break
            e.run(20, ene_every=0)
            x, v = e.coords(0)
            o.set_coords(x, v)
            o.make_pair_lists()


@pytest.mark.parametrize("name", ["golden", "cfg1", "cfg4", "cfg1arqv", "cfg2ar", "cfg1arqvh"])
def test_step_precision_forces(systems, name):
    """The precision of an unrecorded MD step (QGPU_TERMS_STEP_PRECISION: FP32
    bonded, restraint and Q terms from the float coordinates, FP32 energy sums)
    against the FP64 oracle, with the force and energy tolerances above."""
    from qsource_gb300.abi import QGPU_TERMS_STEP_PRECISION
    s = systems[name]
    e = _engine(s)
    e.make_pair_lists()
    d, E, EQ = e.pot_energy(0, terms=0x1F | QGPU_TERMS_STEP_PRECISION)
    o = _oracle(s)
    o.make_pair_lists()
    do, Eo, EQo = o.pot_energy(terms=0x1F)
    assert rel_rms(d, do) <= FORCE_RTOL
    # FP32 pair energies (pp/pw/ww, the FP32 path of every unrecorded step) carry
    # the rounding of each term: about 1e-8 of the sum of |terms|, which for the
    # water sphere of the golden system (ww_el = -7.3 from |terms| summing to
    # 7.7e6 kcal/mol) is 0.02 kcal/mol.
    pair = ["pp_el", "pp_vdw", "pw_el", "pw_vdw", "ww_el", "ww_vdw"]
    assert all(abs(E[k] - Eo[k]) <= max(ENERGY_REL * abs(Eo[k]), STEP_PAIR_ENERGY_ABS) for k in pair)
    assert not energies_close(E, Eo, [k for k in E_KEYS if k not in pair])
    for s_ in range(s.nstates):
        assert not energies_close(EQ[s_], EQo[s_], EQ_KEYS)


def test_run_rows_equals_the_sink(systems):
    """qgpu_run_rows hands over the same records as qgpu_run's callback."""
    from qsource_gb300 import abi
    s = systems["cfg1"]
    a, b = _engine([s, s]), _engine([s, s])
    rows = a.run(20, ene_every=5)
    cap = 16
    E, EQ = (abi.Energies * cap)(), (abi.QEnergy * (cap * abi.MAX_STATES))()
    tr, st = np.zeros(cap, np.int32), np.zeros(cap, np.int32)
    n = b.run_rows(20, 5, E, EQ, tr, st)
    assert n == 8
    for r in range(n):
        step, e, eq = rows[tr[r]][[x[0] for x in rows[tr[r]]].index(st[r])]
        assert E[r].as_dict() == e
        assert [EQ[r * abi.MAX_STATES + k].as_dict() for k in range(s.nstates)] == eq


def test_run_is_bit_deterministic(systems):
    s = systems["cfg2"]
    a = _engine(s)
    a.run(25)
    b = _engine(s)
    b.run(25)
    xa, va = a.coords(0)
    xb, vb = b.coords(0)
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)


def test_batch_equals_single(systems):
    """A trajectory gives bitwise the same result alone or inside a batch."""
    s1, s2 = systems["cfg1"], systems["cfg2"]
    batch = _engine([s1, s2])
    batch.make_pair_lists()
    single = _engine(s2)
    single.make_pair_lists()
    db, Eb, _ = batch.pot_energy(1)
    ds, Es, _ = single.pot_energy(0)
    assert np.array_equal(db, ds)
    assert Eb == Es
    batch.run(12)
    single.run(12)
    assert np.array_equal(batch.coords(1)[0], single.coords(0)[0])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_branches_are_bit_identical(systems, precision):
    """The replayed blocks of a batch split into independent branches (groups
    of consecutive trajectories, qgpu_set_branches) give bitwise the same
    coordinates, velocities and energy records as one branch: 4 trajectories
    of three sizes, 30 steps (three list builds, records every 5 steps)."""
    from qsource_gb300.abi import PRECISION
    batch = [systems["cfg1"], systems["cfg2"], systems["cfg1ar"], systems["cfg2ar"]]
    out = []
    for nb in (1, 4):
        e = _engine(batch)
        e.set_precision(PRECISION[precision])
        e.set_branches(nb)
        # groups of about equal atom counts: at most nb of them
        assert (e.branches() == 1) if nb == 1 else (1 < e.branches() <= nb)
        rows = e.run(30, ene_every=5)
        x, v = e.coords_all()
        out.append((rows, x, v))
    (ra, xa, va), (rb, xb, vb) = out
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)
    assert ra == rb


def test_set_step_moves_the_record_steps(systems):
    """qgpu_set_step sets md_run's step counter on the device (a one-thread
    kernel writes the record window's control words): the same 20 steps run
    from step 100 give records at the same offsets plus 100, and bitwise the
    same coordinates (nothing else of this Berendsen system reads the counter)."""
    out = []
    for start in (0, 100):
        e = _engine([systems["cfg1"]])
        if start:
            e.set_step(start)
        rows = e.run(20, ene_every=5)
        x, v = e.coords_all()
        out.append(([r[0] for r in rows[0]], [r[1] for r in rows[0]], x, v))
    (s0, e0, x0, v0), (s1, e1, x1, v1) = out
    assert len(s0) == 4 and s1 == [k + 100 for k in s0]
    assert e0 == e1
    assert np.array_equal(x0, x1) and np.array_equal(v0, v1)


def test_shake_failure_is_reported(systems):
    """Coincident reference positions make SHAKE diverge: the bounded
    iteration stops at 1000 sweeps and the call returns QGPU_E_SHAKE."""
    from qsource_gb300.engine import QgpuError
    s = systems["cfg1"]
    e = _engine(s)
    xx = s.x.copy()
    o = s.shake_i[0]
    xx[3 * s.shake_j[0]:3 * s.shake_j[0] + 3] = xx[3 * o:3 * o + 3]
    with pytest.raises(QgpuError) as ei:
        e.shake(0, xx, s.x.copy())
    assert ei.value.code == 4
    # the context stays usable once the host hands it valid coordinates again
    e.set_coords(0, s.x, s.v)
    e.make_pair_lists()
    d, _, _ = e.pot_energy(0)
    assert np.isfinite(d).all()


def test_list_overflow_is_reported(systems, monkeypatch):
    from qsource_gb300.engine import QgpuError
    monkeypatch.setenv("QGPU_NB_CAP", "8")
    e = _engine(systems["cfg1"])
    with pytest.raises(QgpuError) as ei:
        e.make_pair_lists()
    assert ei.value.code == 3


def test_invalid_descriptor_is_rejected(systems):
    from qsource_gb300.engine import QgpuError
    import copy
    s = copy.copy(systems["cfg1"])
    s.nstates = 5
    s.lambdas = [0.2] * 5 + [0.0] * 5
    with pytest.raises(QgpuError) as ei:
        _engine(s)
    assert ei.value.code == 6


def test_fep_sums_match_qfep_on_engine_files(engine_lib, tmp_path):
    """Five lambda windows of the 18 A droplet run as one batch with energy
    files attached: the device's streaming FEP sums give qfep's dgf / dgr / dG
    of the files the engine wrote (the oracle's qfep restatement), to 1e-9."""
    from oracle.oracle import qfep_fep
    from qsource_gb300 import synth
    nw, kT, nskip = 5, 0.596163, 2
    systems = [synth.config(1, window=w, lambdas=(1 - w / (nw - 1), w / (nw - 1))) for w in range(nw)]
    e = _engine(systems)
    paths = [str(tmp_path / f"w{w}.en") for w in range(nw)]
    for w, p in enumerate(paths):
        e.ene_open(w, p)
    e.fep_start(list(range(nw)), kT, nskip)
    e.run(200, ene_every=10)
    for w in range(nw):
        e.ene_close(w)
    dgf, dgr, dg, st = e.fep_result()
    of, orr, og, npts = qfep_fep(paths, 2, kT, nskip)
    assert list(npts) == [19] * nw            # frames at steps 10 ... 190
    assert np.all(st[:, 0] == 19 - nskip)
    for a, b in ((dgf, of), (dgr, orr), (dg, og)):
        assert np.allclose(a, b, rtol=1e-9, atol=1e-9), (a, b)


def test_dg_matches_oracle_dynamics(engine_lib):
    """The benchmark metric's qualifier, |dG - oracle| <= 0.1 kcal/mol: five
    lambda windows of the 18 A droplet run 200 steps from the same start on
    the GPU (mixed precision, qfep Part 1 sums on the device from the frames
    at steps 5, 10, ..., 195) and in the FP64 oracle (qfep's Zwanzig sums of
    its own per-step state energies at the same steps)."""
    from qsource_gb300 import synth
    nw, kT, n, every = 5, 0.596163, 200, 5
    systems = [synth.config(1, window=w, lambdas=(1 - w / (nw - 1), w / (nw - 1))) for w in range(nw)]
    e = _engine(systems)
    e.fep_start(list(range(nw)), kT, 0)
    e.run(n, ene_every=every, collect=False)
    _, _, dg, st = e.fep_result()
    V, lam = [], []
    for s in systems:
        o = _oracle(s)
        o.temperature()
        rc, _, oq, _ = o.md_run(n)
        assert rc == 0
        V.append(np.array([[oq[k][i]["total"] for i in range(2)] for k in range(every, n, every)]))
        lam.append(np.array(s.lambdas[:2], dtype=float))
    assert np.all(st[:, 0] == len(V[0]))

    def zwanzig(a, b):
        dv = V[a] @ lam[b] - V[a] @ lam[a]
        return -kT * np.log(np.mean(np.exp(-dv / kT)))
    G = [0.0]
    for w in range(1, nw):
        G.append(G[-1] + 0.5 * (zwanzig(w - 1, w) - zwanzig(w, w - 1)))
    err = np.abs(np.array(G) - dg).max()
    print("dG GPU", np.round(dg, 4).tolist(), "oracle", np.round(G, 4).tolist(), "max |diff|", err)
    assert err <= 0.1


def test_evb_mapping_on_engine_files(engine_lib, tmp_path):
    """Seven windows of a two-state EVB droplet (coupling 15 exp(-0.3 r_12)
    between Q atoms 1 and 2) run as one batch with energy files attached:
    every frame's Hij is A exp(-mu rkl) of its own distance; qfep Parts 1-3
    on the engine's files (qgpu_qfep_evb) equal the numpy restatement of
    qfep, and Part 1 equals the device's streaming FEP sums."""
    from oracle import qfep_ref
    from qsource_gb300 import qfep, synth
    nw, kT, nskip = 7, 0.596163, 4
    qa = synth.neutral_charges(np.random.default_rng(77), 8, 0.5)
    qb = synth.neutral_charges(np.random.default_rng(78), 8, 0.5)
    systems = [synth.synthetic(18.0, 8, 8, np.stack([qa, qb], 1), (1 - w / (nw - 1), w / (nw - 1)), 4100 + w,
                               offdiag=[(1, 2, 1, 2, 15.0, 0.3)]) for w in range(nw)]
    e = _engine(systems)
    paths = [str(tmp_path / f"evb{w}.en") for w in range(nw)]
    for w, p in enumerate(paths):
        e.ene_open(w, p)
    e.fep_start(list(range(nw)), kT, nskip)
    e.run(300, ene_every=5)
    for w in range(nw):
        e.ene_close(w)
    for p in paths:
        _, frames = qfep_ref.read_en(p, 2, 1)
        assert len(frames) == 59
        for _, od in frames:
            (i, j, hij, rkl), = od
            assert (i, j) == (1, 2) and abs(hij - 15.0 * np.exp(-0.3 * rkl)) <= 1e-12 * 15.0
    kw = dict(noffd=1, scale_hij=1.0, nskip=nskip, nbins=10, nmin=3)
    got = qfep.evb(paths, 2, kT, lib=engine_lib, **kw)
    ref = qfep_ref.evb(paths, 2, kT, **kw)
    for key in ("part1", "gap", "part2", "part3"):
        np.testing.assert_allclose(got[key], ref[key], rtol=0, atol=1e-9, err_msg=key)
    dgf, dgr, dg, _ = e.fep_result()
    assert np.allclose(got["part1"][:, 2], dg, rtol=1e-9, atol=1e-9)
    assert (got["part3"][:, 0] >= 3).sum() >= 5


@pytest.mark.parametrize("shape", [[4, 1, 4, 1, 1], [8, 6, 8, 2, 2], [16, 1, 16, 4, 4], [16, 6, 8, 0, 1], [4, 6, 8, 1, 3]])
def test_every_launch_shape_matches_oracle(systems, shape):
    """Each launch shape the autotuner may pick (lanes per water / register
    bound / lanes per solute atom / lanes per Q-water item) gives the oracle's
    forces and energies with the step-precision tolerances."""
    from qsource_gb300.abi import QGPU_TERMS_STEP_PRECISION
    s = systems["cfg2"]
    e = _engine(s)
    e.set_tuning(shape)
    e.make_pair_lists()
    d, E, EQ = e.pot_energy(0, terms=0x1F | QGPU_TERMS_STEP_PRECISION)
    o = _oracle(s)
    o.make_pair_lists()
    do, Eo, EQo = o.pot_energy(terms=0x1F)
    assert rel_rms(d, do) <= FORCE_RTOL
    pair = ["pp_el", "pp_vdw", "pw_el", "pw_vdw", "ww_el", "ww_vdw"]
    assert all(abs(E[k] - Eo[k]) <= max(ENERGY_REL * abs(Eo[k]), STEP_PAIR_ENERGY_ABS) for k in pair)
    for s_ in range(s.nstates):
        assert not energies_close(EQ[s_], EQo[s_], EQ_KEYS)


def test_pipelined_water_loop_is_bit_identical(systems):
    """The software-pipelined neighbour loop (unroll_water 3) visits each
    lane's neighbours in the order of the one-per-iteration loop, so forces
    and energies are bit-identical."""
    from qsource_gb300.abi import QGPU_TERMS_STEP_PRECISION
    out = []
    for uw in (1, 3):
        e = _engine(systems["cfg2"])
        e.set_tuning([4, 6, 8, 1, uw])
        e.make_pair_lists()
        d, E, _ = e.pot_energy(0, terms=0x1F | QGPU_TERMS_STEP_PRECISION)
        out.append((np.array(d), E))
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][1] == out[1][1]


def test_autotune_picks_a_valid_shape_and_is_cached(systems):
    s = systems["cfg1"]
    a = _engine(s)
    t1 = a.autotune()
    assert t1[0] in (4, 8, 16) and t1[1] in (1, 6) and t1[2] in (4, 8, 16) and t1[3] in (1, 2, 4) and t1[4] in (1, 2, 3, 4)
    b = _engine(s)
    assert b.autotune() == t1            # same device and size: the cached choice
    rows = b.run(10, ene_every=5)[0]
    assert len(rows) == 2 and all(np.isfinite(r[1]["potential"]) for r in rows)


# ------------------------------------------------------------- schedule MLP
def _mlp_data(seed, ncurves, kT=0.596, npilot=11, nsamp=20):
    """Pilot statistics of random FEP spread curves (Gaussian model) and the
    true log-spread at the pilot windows."""
    from mlp_ref import pilot_stats, s_curve
    from qsource_gb300.schedule import features
    rng = np.random.default_rng(seed)
    lam = np.linspace(0.0, 1.0, npilot)
    X, Y, curves = [], [], []
    for _ in range(ncurves):
        s = s_curve(rng)
        st = pilot_stats(rng, s, lam, kT, nsamp)
        X.append(features(lam, st, kT))
        Y.append(np.log([s(x) for x in lam]))
        curves.append((s, st))
    return lam, np.concatenate(X), np.concatenate(Y).astype(np.float32), curves


def test_mlp_kernels_match_cpu_reference(engine_lib):
    """One training step of the library's kernels (forward, backward through
    BF16 tensor-core products with FP32 sums) against the CPU reference with
    the same BF16 roundings: loss to 1e-4, each layer's gradient to 1e-2 of its
    norm, predictions to 1e-3."""
    from mlp_ref import forward, loss_and_grad
    from qsource_gb300.schedule import MLP
    rng = np.random.default_rng(11)
    net = MLP(seed=5)
    X = rng.normal(0, 1, (40, 16)).astype(np.float32)
    Y = rng.normal(0, 1, 40).astype(np.float32)
    p0 = net.params.copy()
    ref_loss, ref_grad = loss_and_grad(p0, X, Y)
    pred = net.predict(X)
    assert np.allclose(pred, forward(p0, X)[3][:, 0], rtol=1e-3, atol=1e-3)
    loss, grad = net.train(X, Y, iters=1, lr=0.0)
    assert np.array_equal(net.params, p0)            # lr 0 leaves the parameters
    assert abs(loss[0] - ref_loss) <= 1e-4 * ref_loss
    o = 0
    for n in (128 * 16, 128, 128 * 128, 128, 16 * 128, 16):
        gg, gr = grad[o:o + n].astype(np.float64), ref_grad[o:o + n]
        assert np.linalg.norm(gg - gr) <= 1e-2 * max(np.linalg.norm(gr), 1e-12), o
        o += n


def test_learned_schedule_beats_uniform(engine_lib):
    """Trained on the GPU (the library's kernels) on pilot statistics of
    random spread curves, the network's placement halves (median) the
    expected FEP error of uniform windows on held-out curves (Gaussian gap
    model, 21 windows, equal sampling per window), and does no worse than
    placing by the pilot's own short-run spread."""
    from mlp_ref import schedule_mse
    from qsource_gb300.schedule import MLP, learned_schedule, place
    kT = 0.596
    lam, X, Y, _ = _mlp_data(1, 5)
    net = MLP(seed=2)
    loss, _ = net.train(X, Y, iters=2000, lr=3e-3)
    assert loss[-1] < 0.05 * loss[0]
    lam, _, _, test = _mlp_data(99, 10)
    uni, lrn, raw = [], [], []
    for s, st in test:
        w, _ = learned_schedule(net, lam, st, kT, 21)
        pilot_s = np.sqrt(np.maximum(st[:, 2], st[:, 5])) / (lam[1] - lam[0])
        uni.append(schedule_mse(s, np.linspace(0, 1, 21), kT, 200))
        lrn.append(schedule_mse(s, w, kT, 200))
        raw.append(schedule_mse(s, place(lam, pilot_s, 21), kT, 200))
    assert np.median(np.array(lrn) / np.array(uni)) < 0.5
    assert np.median(np.array(lrn) / np.array(raw)) < 1.05
