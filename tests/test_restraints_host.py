"""The other p_restrain restraints (src/md.f90:15580-15800) in the readers and
the oracle: the [atom_restraints] / [distance_restraints] / [angle_restraints] /
[wall_restraints] sections, and the oracle's forces against central finite
differences of its own restraint energy."""
import copy

import numpy as np


def with_restraints(s, pbc=False):
    """A copy of system s with restraints of every kind (states 0, 1 and 2)."""
    t = copy.copy(s)
    x = np.asarray(s.x).reshape(-1, 3)
    ns = s.nat_solute
    t.rstpos_i = np.array([[0, 0], [1, 1], [ns + 3, 2]], np.int32)
    t.rstpos_x = np.array([list(x[0] + [0.3, -0.2, 0.1]) + [5.0, 6.0, 7.0],
                           list(x[1] + [-0.4, 0.0, 0.2]) + [3.0, 3.0, 3.0],
                           list(x[ns + 3] + [0.5, 0.5, -0.5]) + [2.0, 4.0, 8.0]])
    t.rstdis_i = np.array([[0, 2, 0], [1, ns, 1], [ns, ns + 6, 2]], np.int32)
    t.rstdis_p = np.array([[1.0, 1.5, 10.0], [9.0, 10.0, 4.0], [2.0, 2.5, 6.0]])
    t.rstang_i = np.array([[0, 1, 2, 0], [ns + 1, ns, ns + 2, 1], [2, 0, ns, 2]], np.int32)
    t.rstang_p = np.array([[100.0, 20.0], [90.0, 15.0], [60.0, 5.0]])
    # states beyond the system's own count fall back to state 0 (every state)
    for name in ("rstpos_i", "rstdis_i", "rstang_i"):
        a = getattr(t, name)
        a[a[:, -1] > s.nstates, -1] = 0
    if not pbc:
        t.rstwal_i = np.array([[1, 7, 1], [ns, ns + 29, 0]], np.int32)
        t.rstwal_p = np.array([[0.5, 30.0, 1.5, 0.3], [14.0, 20.0, 2.0, 0.5]])
    return t


def _restraint_energy(o):
    _, E, EQ = o.pot_energy(0x10)
    return E["rst_total"]


def test_oracle_restraint_forces_are_energy_gradients():
    from oracle.oracle import Oracle
    from qsource_gb300 import synth
    s = with_restraints(synth.config(1, lambdas=(0.7, 0.3)))
    o = Oracle(s)
    d, E, EQ = o.pot_energy(0x10)
    assert abs(E["rst_protein"]) > 1.0 and any(abs(q["restraint"]) > 0.1 for q in EQ)
    x0 = np.asarray(s.x, dtype=np.float64).copy()
    atoms = sorted({0, 1, 2, s.nat_solute, s.nat_solute + 1, s.nat_solute + 2, s.nat_solute + 3, s.nat_solute + 6})
    h = 1e-6
    for a in atoms:
        for c in range(3):
            xp, xm = x0.copy(), x0.copy()
            xp[3 * a + c] += h
            xm[3 * a + c] -= h
            o.set_coords(xp)
            ep = _restraint_energy(o)
            o.set_coords(xm)
            em = _restraint_energy(o)
            fd = (ep - em) / (2 * h)
            assert abs(fd - d[3 * a + c]) <= 1e-5 * max(1.0, abs(fd)), (a, c, fd, d[3 * a + c])
        o.set_coords(x0)


def test_restraint_sections_are_read():
    from qsource_gb300.qtop import read_inp
    inp = read_inp("""[atom_restraints]
3 1.0 2.0 3.0 10.0 10.0 5.0 1
[distance_restraints]
1 5 2.0 3.0 10.0 0
[angle_restraints]
1 2 3 109.5 25.0 2
[wall_restraints]
1 46 12.0 20.0 2.0 0.5 1
""")
    assert inp["atom_restraints"] == [[3, 1.0, 2.0, 3.0, 10.0, 10.0, 5.0, 1]]
    assert inp["distance_restraints"] == [[1, 5, 2.0, 3.0, 10.0, 0]]
    assert inp["angle_restraints"] == [[1, 2, 3, 109.5, 25.0, 2]]
    assert inp["wall_restraints"] == [[1, 46, 12.0, 20.0, 2.0, 0.5, 1]]
    assert inp["unsupported"] == []
