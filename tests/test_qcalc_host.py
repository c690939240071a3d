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
