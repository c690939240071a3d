"""qcalc-style analysis on the device (qgpu_calc_*) against the oracle's
restatement of the reference's calc_* modules (oracle/qcalc_ref.py), on frames
of the engine's own MD: the 18 A droplet (sphere) and the reference's PBC
system (box).

Parity unpinned by reference data: the reference ships no qcalc test output,
so these quantities are pinned by the restatement only.

Tolerances: RMSD, centre of mass and geometry 1e-10 relative (FP64 sums in a
different order); RDF bin counts exact (the reference's single-precision
distance and double-precision binning reproduced operation for operation);
centre-of-mass kinetic energies 1e-8 relative (principal axes from a
different eigen-solver); nonbonded LJ and Coulomb sums 1e-10 of (1 + |V|) (FP64 sums of up to 1.6e5
pairs in blocks instead of one running sum)."""
import numpy as np
import pytest

from conftest import golden_system

pytestmark = pytest.mark.gpu


def _frames(s, nframes=6, every=10):
    from qsource_gb300.engine import Engine
    e = Engine(s)
    out = []
    for _ in range(nframes):
        e.run(every)
        x, _ = e.coords(0)
        out.append(x.copy())
    return np.array(out)


@pytest.fixture(scope="module")
def droplet(engine_lib):
    from qsource_gb300 import synth
    s = synth.config(1)
    return s, _frames(s)


def test_rms_com_geom_match_oracle(droplet):
    from oracle import qcalc_ref as ref
    from qsource_gb300.qcalc import Calc
    s, fr = droplet
    c = Calc()
    mask = np.arange(0, s.natom, 7)
    assert np.allclose(c.rms(fr, mask, s.xtop), ref.rms(fr, mask, s.xtop), rtol=1e-10, atol=0)
    mass = np.asarray(s.mass)[np.asarray(s.iac)]
    assert np.allclose(c.com(fr, mask, mass), ref.com(fr, mask, mass), rtol=1e-10, atol=1e-12)
    o = s.nat_solute
    meas = [(0, 1), (o, o + 1), (0, 1, 2), (o + 1, o, o + 2), (0, 1, 2, 3), (4, 5, 6, 7), (o, o + 3, o + 6, o + 9)]
    assert np.allclose(c.geom(fr, meas), ref.geom(fr, meas), rtol=1e-10, atol=1e-9)


def test_com_ke_matches_oracle(droplet):
    """Translational and rotational kinetic energy of the solute's and of a
    water subset's centre of mass over consecutive engine frames (10 steps
    apart)."""
    from oracle import qcalc_ref as ref
    from qsource_gb300.qcalc import Calc
    s, fr = droplet
    mass = np.asarray(s.mass)[np.asarray(s.iac)]
    dt = 20.0                                   # fs between frames (10 steps of 2 fs)
    for mask in (np.arange(s.nat_solute), np.arange(s.nat_solute, s.natom, 5)):
        got = Calc().com_ke(fr, mask, mass, dt)
        want = ref.com_ke(fr, mask, mass, dt)
        assert np.array_equal(got[0], [0.0, 0.0])
        assert np.all(want[1:] > 0)
        assert np.allclose(got, want, rtol=1e-8, atol=0), (got, want)


def test_rmsf_matches_oracle(droplet):
    """RMS fluctuation after every frame (calc_rmsf.f90 RMSF_calc), the value
    qcalc prints per frame: the first frame's is zero, later ones grow with
    the spread of the positions."""
    from oracle import qcalc_ref as ref
    from qsource_gb300.qcalc import Calc
    s, fr = droplet
    mask = np.arange(0, s.natom, 3)
    got = Calc().rmsf(fr, mask)
    want = ref.rmsf(fr, mask)
    assert np.allclose(got, want, rtol=1e-9, atol=1e-12)
    assert abs(got[0]) < 1e-6 and got[-1] > 0


def test_fit_matches_oracle(droplet):
    """Least-squares fit of the solute (calc_fit.f90): the engine's frames and
    rigidly moved copies of the topology coordinates (fitted back onto them
    to 1e-9 A), against the restatement."""
    from oracle import qcalc_ref as ref
    from qsource_gb300.qcalc import Calc
    s, fr = droplet
    ns = int(s.nat_solute)
    mass = np.asarray(s.mass)[np.asarray(s.iac)]
    mask = np.arange(ns)
    got, st = Calc().fit(fr, ns, mask, mass, s.xtop)
    want, wst = ref.fit(fr, ns, mask, mass, s.xtop)
    assert np.array_equal(st, wst)
    assert np.abs(got - want).max() < 1e-9
    # rigid copies of the reference come back onto it
    rng = np.random.default_rng(9)
    x0 = np.asarray(s.xtop).reshape(-1, 3)
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, a, b, c = q
    R = np.array([[1 - 2 * (b * b + c * c), 2 * (a * b - c * w), 2 * (a * c + b * w)],
                  [2 * (a * b + c * w), 1 - 2 * (a * a + c * c), 2 * (b * c - a * w)],
                  [2 * (a * c - b * w), 2 * (b * c + a * w), 1 - 2 * (a * a + b * b)]])
    moved = x0.copy()
    moved[:ns] = x0[:ns] @ R.T + np.array([3.0, -2.0, 7.5])
    back, st2 = Calc().fit(moved.ravel()[None, :], ns, mask, mass, s.xtop)
    assert st2[0] == 0
    assert np.abs(back.reshape(-1, 3)[:ns] - x0[:ns]).max() < 1e-9


def test_rdf_counts_match_oracle_sphere(droplet):
    from oracle import qcalc_ref as ref
    from qsource_gb300.qcalc import Calc
    s, fr = droplet
    ox = np.arange(s.nat_solute, s.natom, 3)
    got = Calc().rdf_counts(fr, ox, ox, 12.0, 120)
    assert np.array_equal(got, ref.rdf_counts(fr, ox, ox, 12.0, 120))
    assert got.sum() > 0


def test_rdf_counts_match_oracle_box(engine_lib):
    from oracle import qcalc_ref as ref
    from qsource_gb300.qcalc import Calc
    s = golden_system("basic_pbc")
    fr = np.array([s.x])
    ox = np.arange(s.nat_solute, s.natom, 3)[:1500]
    lig = np.arange(0, s.nat_solute)
    for m1, m2 in ((ox, ox), (lig, ox)):
        got = Calc().rdf_counts(fr, m1, m2, 15.0, 150, box=s.boxlength)
        assert np.array_equal(got, ref.rdf_counts(fr, m1, m2, 15.0, 150, box=s.boxlength))


def test_analysis_of_a_dcd_written_from_engine_frames(droplet, tmp_path):
    """Frames through the reference's DCD layout (single precision) and back."""
    from oracle import qcalc_ref as ref
    from qsource_gb300.qcalc import Calc, read_dcd, write_dcd
    s, fr = droplet
    p = str(tmp_path / "traj.dcd")
    write_dcd(p, fr, interval=10)
    head, back = read_dcd(p)
    assert head["n_frames"] == len(fr) and back.shape == fr.shape
    mask = np.arange(s.natom)
    assert np.allclose(Calc().rms(back, mask, s.xtop), ref.rms(back, mask, s.xtop), rtol=1e-10, atol=0)


def test_nb_energies_match_oracle_reference_topology(engine_lib):
    """calc_nb on the reference's own topology: the solute against every atom
    (overlapping masks, angle pairs dropped, 1-4 pairs), three perturbed
    frames."""
    from oracle import qcalc_ref as ref
    from qsource_gb300.qcalc import Calc, nb_make_list
    g = golden_system("basic_sph")
    rng = np.random.default_rng(9)
    x0 = np.asarray(g.x, dtype=np.float64)
    fr = np.array([x0 + rng.normal(0, 0.05, x0.shape) for _ in range(3)])
    lst = nb_make_list(g, np.arange(g.nat_solute), np.arange(g.natom))
    assert len(lst.pairs) > 150000
    got = Calc().nb(fr, lst)[:, 0]
    want = ref.nb_calc(fr, lst.pairs, lst.AA, lst.BB, lst.qq)
    assert np.all(np.abs(got - want) <= 1e-10 * (1 + np.abs(want))), (got, want)


def test_nb_energies_fep_both_rules_match_oracle(engine_lib):
    """The per-state form (Q atoms at their states' types and charges,
    weighted by lambda) under both combination rules, with a pair of
    coincident atoms in one frame (r = 0 adds nothing)."""
    from oracle import qcalc_ref as ref
    from qsource_gb300 import synth
    from qsource_gb300.qcalc import Calc, nb_make_list
    rng = np.random.default_rng(5)
    qa = synth.neutral_charges(rng, 6, 0.4)
    for rule in (1, 2):
        g = synth.synthetic(8.0, 24, 6, np.stack([qa, -qa], 1), (0.5, 0.5), 11, vdw_rule=rule, qvdw=True)
        nsol = int(g.nat_solute)
        q = np.flatnonzero(np.asarray(g.iqatom)[:nsol] >= 0)
        m2 = np.arange(g.natom)
        x0 = np.asarray(g.x, dtype=np.float64)
        fr = np.array([x0 + rng.normal(0, 0.05, x0.shape) for _ in range(2)])
        w = nsol + 4
        fr[1, 3 * w:3 * w + 3] = fr[1, 3 * q[0]:3 * q[0] + 3]
        lst = nb_make_list(g, q, m2, fep=True)
        lam = np.array([0.3, 0.7])
        got = Calc().nb(fr, lst, lam)[:, 0]
        want = ref.nb_calc(fr, lst.pairs, lst.AA, lst.BB, lst.qq, lambdas=lam, arith=lst.arith)
        assert np.all(np.isfinite(got))
        assert np.all(np.abs(got - want) <= 1e-10 * (1 + np.abs(want))), (rule, got, want)


def test_nb_empty_list(engine_lib):
    """One atom in both masks: the overlap rule leaves no pair, zero energies."""
    from qsource_gb300.qcalc import Calc, nb_make_list
    g = golden_system("basic_sph")
    lst = nb_make_list(g, [3], [3])
    assert len(lst.pairs) == 0
    got = Calc().nb(np.array([g.x, g.x]), lst)
    assert np.array_equal(got, np.zeros((2, 1, 2)))


def test_nb_residue_lists_match_oracle(engine_lib):
    """nb_qp: one list per residue against the Q-atom mask (here the first
    60 water molecules as residues against the 46 Q atoms of the reference's
    topology), all lists summed in one call, and the per-residue averages over
    the frames."""
    from oracle import qcalc_ref as ref
    from qsource_gb300.qcalc import Calc, nb_averages, nb_qp_make_lists
    g = golden_system("basic_sph")
    nsol = int(g.nat_solute)
    rng = np.random.default_rng(4)
    x0 = np.asarray(g.x, dtype=np.float64)
    fr = np.array([x0 + rng.normal(0, 0.05, x0.shape) for _ in range(4)])
    residues = [np.arange(nsol + 3 * w, nsol + 3 * w + 3) for w in range(60)]
    qmask = np.arange(nsol)
    lst = nb_qp_make_lists(g, residues, qmask)
    assert len(lst.starts) == 61 and lst.starts[-1] == 60 * 3 * nsol
    got = Calc().nb(fr, lst)
    want = ref.nb_qp(fr, g, residues, qmask)
    assert got.shape == want.shape == (4, 60, 2)
    assert np.all(np.abs(got - want) <= 1e-10 * (1 + np.abs(want)))
    for r in (0, 17, 59):
        for e in (0, 1):
            a, b = nb_averages(got[:, r, e]), ref.nb_averages(want[:, r, e])
            assert abs(a - b) <= 1e-10 * (1 + abs(b))
