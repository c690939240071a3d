"""Host side of the qcalc-style analysis: the DCD layout of src/trj.f90 and the
oracle's calc_geom / calc_rdf restatements on configurations with known answers
(parity unpinned by reference data: the reference ships no qcalc test output)."""
import math
import struct

import numpy as np


def test_dcd_round_trip_and_layout(tmp_path):
    from qsource_gb300.qcalc import read_dcd, write_dcd
    rng = np.random.default_rng(3)
    frames = rng.normal(0, 10, size=(4, 3 * 7))
    p = str(tmp_path / "t.dcd")
    write_dcd(p, frames, interval=25, n_degf=12, topology="lig_w.top")
    head, back = read_dcd(p)
    assert head["n_frames"] == 4 and head["interval"] == 25 and head["n_steps"] == 100 and head["n_degf"] == 12
    assert head["atoms"] == 7 and head["mask_rows"] == ["all"] and head["topology"] == "lig_w.top"
    assert np.array_equal(back, frames.astype(np.float32).astype(np.float64))
    raw = open(p, "rb").read()
    # record 1: 84-byte payload starting with CORD; record 3: the atom count
    assert struct.unpack("<i", raw[:4])[0] == 84 and raw[4:8] == b"CORD"
    off = 8 + 84 + 4 + 4 + 3 * 80 + 4
    assert struct.unpack("<iii", raw[off:off + 12]) == (4, 7, 4)


def test_geom_known_answers():
    from oracle.qcalc_ref import geom
    # atoms: 0 (1,0,0), 1 (0,0,0), 2 (0,1,0), 3 (0,1,1): angle 0-1-2 = 90, torsion 0-1-2-3 = +-90
    x = np.array([[1, 0, 0], [0, 0, 0], [0, 1, 0], [0, 1, 1]], dtype=np.float64).reshape(1, -1)
    g = geom(x, [(0, 1), (0, 1, 2), (0, 1, 2, 3), (0, 2)])
    assert g[0, 0] == 1.0 and abs(g[0, 1] - 90.0) < 1e-12 and abs(abs(g[0, 2]) - 90.0) < 1e-12
    assert abs(g[0, 3] - math.sqrt(2.0)) < 1e-15


def test_rdf_counts_known_answers():
    from oracle.qcalc_ref import rdf_counts
    # three atoms on a line 1 A apart: pairs (0,1) 1 A, (0,2) 2 A, (1,2) 1 A, both orders
    x = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0]], dtype=np.float64).reshape(1, -1)
    c = rdf_counts(x, [0, 1, 2], [0, 1, 2], radius=4.0, nbins=4)
    assert list(c) == [0, 4, 2, 0]
    # in a 3 A box the (0, 2) pair is 1 A apart through the boundary
    c = rdf_counts(x, [0, 1, 2], [0, 1, 2], radius=4.0, nbins=4, box=[3.0, 3.0, 3.0])
    assert list(c) == [0, 6, 0, 0]


def test_rmsf_known_answer():
    """Two atoms alternating between two positions 2 A apart along x: after
    an even number of frames each atom's fluctuation is 1 A."""
    from oracle import qcalc_ref as ref
    frames = np.zeros((4, 2, 3))
    frames[0::2, :, 0] = 0.0
    frames[1::2, :, 0] = 2.0
    got = ref.rmsf(frames.reshape(4, -1), [0, 1])
    assert got[0] == 0.0
    assert abs(got[1] - 1.0) < 1e-12 and abs(got[3] - 1.0) < 1e-12


def _rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def test_fit_known_answer():
    """Frames that are rigid rotations and translations of the reference are
    fitted back onto it exactly; solvent atoms are left alone."""
    from oracle import qcalc_ref as ref
    rng = np.random.default_rng(5)
    nsol, natom = 12, 15
    xref = rng.normal(0, 3, size=(natom, 3))
    mass = rng.uniform(1, 16, size=natom)
    frames = []
    for _ in range(3):
        R, t = _rotation(rng), rng.normal(0, 5, size=3)
        fr = xref.copy()
        fr[:nsol] = xref[:nsol] @ R.T + t
        frames.append(fr.ravel())
    out, st = ref.fit(np.array(frames), nsol, np.arange(0, nsol, 2), mass, xref.ravel())
    assert np.array_equal(st, [0, 0, 0])
    for f in range(3):
        got = out[f].reshape(-1, 3)
        assert np.abs(got[:nsol] - xref[:nsol]).max() < 1e-10
        assert np.array_equal(got[nsol:], np.array(frames[f]).reshape(-1, 3)[nsol:])


def _nb_system(vdw_rule=1, qvdw=True):
    """A seeded synthetic droplet with two Q states (per-state Q types and
    charges) and the chain's consecutive-atom angles added (the synthetic
    topology has none), so every rule of the nonbond list is exercised."""
    from qsource_gb300 import synth
    rng = np.random.default_rng(5)
    qa = synth.neutral_charges(rng, 6, 0.4)
    g = synth.synthetic(8.0, 24, 6, np.stack([qa, -qa], 1), (0.5, 0.5), 11, vdw_rule=vdw_rule, qvdw=qvdw)
    n = int(g.nat_solute)
    g.ang = np.array([(i, i + 1, i + 2, 1) for i in range(0, n - 2, 3)], dtype=np.int32)
    return g


def _same_list(a, b):
    pa, A, B, Q = b
    assert np.array_equal(a.pairs.astype(np.int64), pa)
    for x, y in ((a.AA, A), (a.BB, B), (a.qq, Q)):
        assert x.shape == y.shape and np.array_equal(x, y)


def test_nb_list_matches_restatement_on_reference_topology():
    """The reference's own topology (46 solute atoms with angles and 1-4
    pairs): solute against solute and 150 water atoms (overlapping masks)."""
    from conftest import golden_system
    from oracle import qcalc_ref as ref
    from qsource_gb300.qcalc import nb_make_list
    g = golden_system("basic_sph")
    nsol = int(g.nat_solute)
    m1 = np.arange(nsol)
    m2 = np.concatenate([np.arange(nsol), np.arange(nsol, nsol + 150)])
    got = nb_make_list(g, m1, m2)
    want = ref.nb_make_list(g, m1, m2)
    _same_list(got, want)
    # the overlap's pairs once each; angle pairs dropped; 1-4 pairs at el14 scale
    n_self = nsol * (nsol - 1) // 2
    ang = {tuple(sorted(p)) for a in np.asarray(g.ang)[:, :3] for p in ((a[0], a[1]), (a[0], a[2]), (a[1], a[2]))}
    assert len(got.pairs) == n_self - len(ang) + nsol * 150
    assert not {tuple(sorted(p)) for p in got.pairs.tolist()} & ang


def test_nb_list_fep_geometric_and_arithmetic_match_restatement():
    from oracle import qcalc_ref as ref
    from qsource_gb300.qcalc import nb_make_list
    for rule in (1, 2):
        g = _nb_system(vdw_rule=rule)
        nsol = int(g.nat_solute)
        q = np.flatnonzero(np.asarray(g.iqatom)[:nsol] >= 0)
        m2 = np.concatenate([np.arange(nsol), np.arange(nsol, nsol + 30)])
        for fep in (False, True):
            got = nb_make_list(g, q, m2, fep=fep)
            assert got.arith == (rule == 2)
            _same_list(got, ref.nb_make_list(g, q, m2, fep=fep))
            assert got.AA.shape[1] == (2 if fep else 1)


def test_nb_energy_known_answers():
    from oracle import qcalc_ref as ref
    # atoms 0 and 1 two A apart, atom 2 on top of atom 0 (r = 0 adds nothing)
    x = np.array([[0, 0, 0], [2, 0, 0], [0, 0, 0]], dtype=np.float64).reshape(1, -1)
    pairs = np.array([[0, 1], [0, 2]])
    A, B, Q = np.array([[3.0], [7.0]]), np.array([[5.0], [7.0]]), np.array([[11.0], [7.0]])
    v = ref.nb_calc(x, pairs, A, B, Q)
    assert np.allclose(v[0], [3.0 / 4096 - 5.0 / 64, 5.5], rtol=1e-15, atol=0)
    # arithmetic rule: sqrt(BB)*AA^6/r^6*(AA^6/r^6 - 2) is -sqrt(BB) at r = AA
    va = ref.nb_calc(x, pairs[:1], np.array([[2.0]]), np.array([[0.25]]), np.array([[0.0]]), arith=True)
    assert abs(va[0, 0] + 0.5) < 1e-15
    # two states weighted by lambda
    v2 = ref.nb_calc(x, pairs[:1], np.array([[3.0, 0.0]]), np.array([[5.0, 0.0]]), np.array([[11.0, 1.0]]),
                     lambdas=[0.25, 0.75])
    assert np.allclose(v2[0], [0.25 * (3.0 / 4096 - 5.0 / 64), 0.25 * 5.5 + 0.75 * 0.5], rtol=1e-15, atol=0)
    from qsource_gb300.qcalc import nb_averages
    assert nb_averages([1.0, 2.0, 3.0, 4.0]) == ref.nb_averages([1.0, 2.0, 3.0, 4.0]) == 2.5


def test_com_ke_known_answers():
    """A rectangle of four equal masses, (+-a, 0, 0) and (0, +-b, 0), turned by
    theta about z between frames: the centre stays put (no translational
    energy) and the three principal axes give L^2/(2I) = m s^2 (a^2 + b^2),
    m s^2 b^2 and m s^2 a^2 per dt^2 (s = sin theta), so the rotational energy
    is 2 m s^2 (a^2 + b^2)/dt^2 * 2390.  The same body moved by d per frame
    has 0.5 M |d|^2/dt^2 * 2390 and no rotation.  Frame 0 gives zeros."""
    from oracle import qcalc_ref as ref
    m, a, b, th, dt = 12.0, 1.5, 0.8, 0.01, 2.0
    x0 = np.array([[a, 0, 0], [-a, 0, 0], [0, b, 0], [0, -b, 0]])
    R = np.array([[math.cos(th), -math.sin(th), 0], [math.sin(th), math.cos(th), 0], [0, 0, 1]])
    frames = np.array([x0.ravel(), (x0 @ R.T).ravel()])
    v = ref.com_ke(frames, [0, 1, 2, 3], np.full(4, m), dt)
    assert np.array_equal(v[0], [0.0, 0.0])
    want = 2 * m * math.sin(th) ** 2 * (a * a + b * b) / dt ** 2 * 2390
    assert abs(v[1, 0]) < 1e-20 and abs(v[1, 1] - want) < 1e-12 * want
    d = np.array([0.3, -0.1, 0.2])
    frames = np.array([x0.ravel(), (x0 + d).ravel()])
    v = ref.com_ke(frames, [0, 1, 2, 3], np.full(4, m), dt)
    assert abs(v[1, 0] - 0.5 * 4 * m * float(d @ d) / dt ** 2 * 2390) < 1e-12 and abs(v[1, 1]) < 1e-20
