"""Seeded synthetic water-sphere systems in Q's own topology/FEP/input form.

The generator writes the same dicts that :mod:`qsource_gb300.qtop` reads from
.top/.fep/.inp files, so every synthetic system passes through the same
start-up path (:func:`qsource_gb300.system.build`) as a reference input.

Recipe (stated, seeded; no public data set is involved):
  * water: TIP3P (O -0.834 e, H +0.417 e, O-H 0.9572 A, HOH 104.52 deg) on a
    jittered cubic lattice at 0.0334 molecules/A^3 (spacing 3.104 A, uniform
    jitter +-0.25 A), uniform random orientations, O inside the sphere radius;
  * solute: a self-avoiding chain with 1.53 A harmonic bonds (k = 300
    kcal/mol/A^2), four OPLS LJ types, charges N(0, sigma) neutralised, charge
    groups of 4 consecutive atoms (switch atom = first), 1-2/1-3 exclusions
    and 1-4 pairs along the chain;
  * Q region: the first nq chain atoms (at the sphere centre) with per-state
    charge sets; the LJ types do not change between states.
LJ parameters are the Q-OPLSAA values (sqrt(A), sqrt(B) per code) for OW, HW,
CT, CA, N and O.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.spatial import cKDTree

from .system import System, build

# name: (Avdw1, Avdw2, Bvdw1, Avdw3, Bvdw2&3, mass)
OPLS = {
    "OW": (762.89, 762.89, 24.39, 539.45, 17.25, 16.00),
    "HW": (0.0, 0.0, 0.0, 0.0, 0.0, 1.008),
    "CT": (944.52, 944.52, 22.03, 667.88, 15.58, 12.01),
    "CA": (1059.13, 1059.13, 23.67, 748.92, 16.74, 12.01),
    "N": (971.75, 971.75, 28.31, 687.13, 20.02, 14.01),
    "O": (616.44, 616.44, 23.77, 435.89, 16.81, 16.00),
}
TYPES = ["OW", "HW", "CT", "CA", "N", "O"]
R_OH, ANG_HOH = 0.9572, 104.52
DENSITY = 0.0334
BOND = 1.53


def _chain(n: int, R: float, rng: np.random.Generator) -> np.ndarray:
    """Self-avoiding random chain of n atoms starting at the origin."""
    pos = np.zeros((max(n, 1), 3))
    if n <= 1:
        return pos[:n]
    k = 1
    tries = 0
    while k < n:
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        p = pos[k - 1] + BOND * d
        if np.linalg.norm(p) > R - 4.0:
            p = pos[k - 1] + BOND * (0.3 * d - 0.7 * pos[k - 1] / np.linalg.norm(pos[k - 1]))
            p = pos[k - 1] + BOND * (p - pos[k - 1]) / np.linalg.norm(p - pos[k - 1])
        ok = True
        if k >= 2:
            dist = np.linalg.norm(pos[: k - 1] - p, axis=1)
            ok = dist.min() >= 2.6
        if ok:
            pos[k] = p
            k += 1
            tries = 0
        else:
            tries += 1
            if tries > 200:        # back off a few atoms and regrow
                k = max(1, k - 5)
                tries = 0
    return pos


def _waters(R: float, solute: np.ndarray, rng: np.random.Generator, box: float = 0.0) -> np.ndarray:
    """Water O on a jittered lattice inside the sphere of radius R, or filling
    the periodic cube of side `box` (a whole number of lattice cells, so the
    lattice continues across the faces), with random orientations; waters
    closer than 2.6 A to the solute are left out."""
    a = (1.0 / DENSITY) ** (1.0 / 3.0)
    if box > 0.0:
        m = int(round(box / a))
        g = (np.arange(m) + 0.5) * (box / m) - 0.5 * box
        O = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
        O = O + rng.uniform(-0.25, 0.25, size=O.shape)
    else:
        m = int(math.ceil(R / a)) + 1
        g = np.arange(-m, m + 1) * a
        O = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
        O = O + rng.uniform(-0.25, 0.25, size=O.shape)
        O = O[np.linalg.norm(O, axis=1) <= R]
    # random orientations: uniform unit quaternions
    q = rng.normal(size=(len(O), 4))
    q /= np.linalg.norm(q, axis=1)[:, None]
    w, x, y, z = q.T
    Rm = np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], 1)
    h = math.radians(ANG_HOH) / 2
    loc = np.array([[0, 0, 0], [R_OH * math.sin(h), 0, R_OH * math.cos(h)], [-R_OH * math.sin(h), 0, R_OH * math.cos(h)]])
    W = O[:, None, :] + np.einsum("nij,aj->nai", Rm, loc)
    if len(solute):
        tree = cKDTree(solute, boxsize=None)
        Wq = W.reshape(-1, 3)
        if box > 0.0:   # minimum image: solute images across the faces count
            Wq = Wq - box * np.round(Wq / box)
        d, _ = tree.query(Wq)
        keep = d.reshape(-1, 3).min(axis=1) >= 2.6
        W = W[keep]
    return W.reshape(-1, 3)


def synthetic(R: float, n_solute: int, nq: int, qcharges: np.ndarray, lambdas, seed: int, *,
              solute_sigma: float = 0.3, T: float = 300.0, stepsize: float = 1.0, tau_T: float = 100.0,
              NBcycle: int = 10, Rc: float = 10.0, offdiag=None, initial_velocities: bool = True,
              any_atom: bool = False, vdw_rule: int = 1, qvdw: bool = False, q_lj_scale=(0.9, 0.5),
              solute_restraint: float = 0.0, box: float = 0.0, water_h_lj: bool = False) -> System:
    """Water sphere of radius R around a solute chain of n_solute atoms whose
    first nq atoms are Q atoms with per-state charges qcharges[nq, nstates].

    vdw_rule 2 gives the same LJ types in the arithmetic combination rule
    (ivdw_rule 2).  qvdw gives the Q atoms their own per-state Q types
    ([atom_types] / [change_atoms] of the FEP file): state 1 the CT type,
    the other states a softer copy (sqrt(A) and sqrt(B) of the CT type scaled
    by q_lj_scale; (0, 0) makes the Q atoms vanish from the LJ terms in those
    states, the end-point case of a decoupling free energy).

    solute_restraint > 0 adds a sequence restraint ([sequence_restraints] of
    the .inp: atoms 1..n_solute, centre to the centre of the topology
    positions) with that force constant in kcal/(mol A^2), which keeps a small
    solute inside the droplet over long runs; without it a neutral chain can
    leave the sphere (nothing restrains the solute).

    water_h_lj (arithmetic rule only) gives the water hydrogens LJ parameters.

    box > 0 builds a periodic cube of that side instead of the sphere: waters
    fill it, the chain grows within R of its centre, the Q switching atom is
    the first Q atom, and the solvent is put back in the box at each list
    update (R must stay below box / 2 minus the cut-off).

    any_atom selects the any-atom cut-off for the solute charge groups
    (topology flag iuse_switch_atom = 0).  The chain's groups are 4
    consecutive atoms with no angle terms, so two atoms of groups whose
    switch atoms lie beyond the cut-off can come within 2 A of each other with
    no LJ repulsion between them under the switch-atom cut-off; the solute
    systems of the benchmark use the any-atom cut-off for that reason."""
    rng = np.random.default_rng(seed)
    S = qcharges.shape[1]
    n_solute = max(n_solute, nq)
    chain = _chain(n_solute, R, rng)
    W = _waters(R, chain, rng, box)
    nw = len(W) // 3
    natom = n_solute + 3 * nw
    xtop = np.concatenate([chain.reshape(-1), W.reshape(-1)])
    stype = rng.integers(2, 6, size=n_solute)          # CT CA N O (0-based into TYPES)
    iac = np.concatenate([stype + 1, np.tile([1, 2, 2], nw)]).astype(np.int32)
    crg = np.zeros(natom)
    if n_solute > nq:
        c = rng.normal(0.0, solute_sigma, size=n_solute - nq)
        crg[nq:n_solute] = c - c.mean()
    crg[:nq] = qcharges[:, 0]
    crg[n_solute:] = np.tile([-0.834, 0.417, 0.417], nw)
    # bonds: chain + water (O-H1, O-H2, H1-H2)
    hh = 2 * R_OH * math.sin(math.radians(ANG_HOH) / 2)
    bnd = [(i + 1, i + 2, 1) for i in range(n_solute - 1)]
    for w in range(nw):
        o = n_solute + 3 * w + 1
        bnd += [(o, o + 1, 2), (o, o + 2, 2), (o + 1, o + 2, 3)]
    bondlib = np.array([[300.0, BOND], [1106.0, R_OH], [0.0, hh]])
    # charge groups
    first, last, sw, atoms = [], [], [], []
    for g0 in range(0, n_solute, 4):
        members = list(range(g0 + 1, min(g0 + 4, n_solute) + 1))
        first.append(len(atoms) + 1); atoms += members; last.append(len(atoms)); sw.append(members[0])
    ncgp_solute = len(first)
    for w in range(nw):
        o = n_solute + 3 * w + 1
        first.append(len(atoms) + 1); atoms += [o, o + 1, o + 2]; last.append(len(atoms)); sw.append(o)
    ex = [(i, i + 1) for i in range(1, n_solute)] + [(i, i + 2) for i in range(1, n_solute - 1)]
    p14 = [(i, i + 3) for i in range(1, n_solute - 2)]
    av = np.array([[OPLS[t][0], OPLS[t][1], OPLS[t][3]] for t in TYPES])
    bv = np.array([[OPLS[t][2], OPLS[t][4], OPLS[t][4]] for t in TYPES])
    if vdw_rule == 2:
        av, bv = _arithmetic_params(av, bv)
        if water_h_lj:
            # water hydrogens with LJ (R*/2 = 0.2245 A, eps = 0.046 kcal/mol in
            # every code), the case nonbon2_ww / nonbon2_qw take on all atoms
            hw = TYPES.index("HW")
            av[hw, :] = 0.2245
            bv[hw, :] = math.sqrt(0.046)
    top = {
        "version": 5.06, "ff_type": 2, "natom": natom, "nat_solute": n_solute, "solv_atom": 3,
        "xtop": xtop, "iac": iac,
        "nbonds_solute": max(0, n_solute - 1), "bnd": np.array(bnd, dtype=np.int32).reshape(-1, 3), "bondlib": bondlib,
        "nangles_solute": 0, "ang": np.zeros((0, 4), np.int32), "anglib": np.zeros((0, 4)),
        "ntors_solute": 0, "tor": np.zeros((0, 5), np.int32), "torlib": np.zeros((0, 4)),
        "nimps_solute": 0, "imp": np.zeros((0, 5), np.int32), "imp_type": 2, "implib": np.zeros((0, 2)),
        "crg": crg, "ncgp_solute": ncgp_solute, "iuse_switch_atom": 0 if any_atom else 1,
        "cgp_first": np.array(first, np.int32), "cgp_last": np.array(last, np.int32),
        "cgp_switch": np.array(sw, np.int32), "cgpatom": np.array(atoms, np.int32),
        "ivdw_rule": vdw_rule, "el14_scale": 0.5, "coulomb_constant": 332.0,
        "mass": np.array([OPLS[t][5] for t in TYPES]), "avdw": av, "bvdw": bv,
        "lj2": np.zeros((0, 2), np.int32),
        "list14": np.array(p14, np.int32).reshape(-1, 2), "list14long": np.zeros((0, 2), np.int32),
        "listex": np.array(ex, np.int32).reshape(-1, 2), "listexlong": np.zeros((0, 2), np.int32),
        "istart_mol": np.array([1] + [n_solute + 3 * w + 1 for w in range(nw)], np.int32),
        "solvent_type": 0, "rexcl_o": R + 2.0, "rwat": R,
        "xpcent": np.zeros(3), "xwcent": np.zeros(3), "nexats": 0, "nexwat": 0,
        "excl": np.zeros(natom, np.uint8),
        "nres": 1 + nw, "nres_solute": 1,
    }
    if box > 0.0:
        top.update({"use_pbc": True, "boxlength": np.full(3, float(box)), "boxcentre": np.zeros(3)})
    atom_types, change_atoms = [], []
    if qvdw:
        ct = TYPES.index("CT")
        hard = [av[ct, 0] ** 2, bv[ct, 0] ** 2, av[ct, 1] ** 2, bv[ct, 1] ** 2, av[ct, 2] ** 2, bv[ct, 2] ** 2]
        if vdw_rule == 2:
            hard = [av[ct, 0], bv[ct, 0], av[ct, 1], bv[ct, 1], av[ct, 2], bv[ct, 2]]
        # [atom_types] rows hold the parameters as the topology does (sqrt(A), sqrt(B) per code)
        hard = [math.sqrt(v) for v in hard] if vdw_rule == 1 else hard
        soft = [v * (q_lj_scale[1] if k % 2 else q_lj_scale[0]) for k, v in enumerate(hard)]
        atom_types = [("Qhard", hard, 12.011), ("Qsoft", soft, 12.011)]
        change_atoms = [(i + 1, ["Qhard"] + ["Qsoft"] * (S - 1)) for i in range(nq)]
    fep = {
        "nstates": S, "iqseq": np.arange(1, nq + 1, dtype=np.int32),
        "change_charges": [(i + 1, list(qcharges[i])) for i in range(nq)],
        "atom_types": atom_types, "change_atoms": change_atoms, "soft_pairs": [], "el_scale": [], "excluded_pairs": [],
        "bond_types": {}, "change_bonds": [], "angle_types": {}, "change_angles": [],
        "torsion_types": {}, "change_torsions": [], "improper_types": {}, "change_impropers": [],
        "off_diagonals": list(offdiag or []), "unsupported": [],
        "qswitch": 1 if box > 0.0 and nq else None,
    }
    inp = {
        "steps": 0, "stepsize": stepsize, "temperature": T, "bath_coupling": tau_T, "thermostat": "berendsen",
        "integrator": "leap-frog", "separate_scaling": True, "random_seed": seed, "initial_temperature": T,
        "shake_solvent": True, "shake_solute": False, "shake_hydrogens": False, "lrf": True,
        "Rcpp": Rc, "Rcww": Rc, "Rcpw": Rc, "Rcq": 99.0, "RcLRF": 99.0,
        "shell_radius": None, "shell_force": 10.0, "excluded_force": 200.0, "solvent_radius": None,
        "radial_force": -1.0, "polarisation": False, "morse_depth": -1.0, "morse_width": -1.0,
        "non_bond": NBcycle, "lambdas": list(lambdas), "topology": None, "fep": None, "unsupported": [],
        "sequence_restraints": [(1, n_solute, solute_restraint, 0, 1)] if solute_restraint > 0 else [],
        "pbc": box > 0.0, "put_solvent_back_in_box": box > 0.0,
    }
    s = build(top, fep, inp)
    if initial_velocities:
        m = s.mass[s.iac]
        sd = np.sqrt(0.001986 * T / m)
        s.v = (rng.normal(size=(natom, 3)) * sd[:, None]).reshape(-1)
    return s


def _arithmetic_params(av: np.ndarray, bv: np.ndarray):
    """The same LJ types for the arithmetic combination rule (ivdw_rule 2):
    from sqrt(A) = av, sqrt(B) = bv of V = A/r^12 - B/r^6 per type, the
    radius R* = 2^(1/6) sigma / 2 with sigma^6 = A/B and sqrt(eps) with
    eps = B^2 / (4 A), so that eps_ij (R*_i + R*_j)^12 / r^12 - 2 eps_ij
    (R*_i + R*_j)^6 / r^6 reproduces the type's own LJ curve (zero for types
    without LJ)."""
    A, B = av ** 2, bv ** 2
    with np.errstate(divide="ignore", invalid="ignore"):
        sig6 = np.where(B > 0, A / np.where(B > 0, B, 1.0), 0.0)
        eps = np.where(A > 0, B ** 2 / (4.0 * np.where(A > 0, A, 1.0)), 0.0)
    rstar = 0.5 * 2.0 ** (1.0 / 6.0) * sig6 ** (1.0 / 6.0)
    return rstar, np.sqrt(eps)


def neutral_charges(rng: np.random.Generator, n: int, sigma: float) -> np.ndarray:
    c = rng.normal(0.0, sigma, size=n)
    return c - c.mean()


def config(cfg: int, replica: int = 0, window: int = 0, nwindows: int = 21, **kw) -> System:
    """The benchmark systems (seed = 1000*cfg + 100*replica + window).

    1: R 18 A, 8 Q atoms (the whole solute), 2 states, lambda (0.5, 0.5)
    2: R 30 A, 2,000-atom chain, 50 Q atoms, 2 states
    4: R 35 A, 3,000-atom chain, 30 Q atoms, 4 EVB states, Hij = 20 kcal/mol
    5: R 40 A, 4,000-atom chain, 60 Q atoms, 2 states
    """
    seed = 1000 * cfg + 100 * replica + window
    qrng = np.random.default_rng(1000 * cfg)         # Q charges shared by all windows of a config
    if cfg == 1:
        qa = neutral_charges(qrng, 8, 0.4)
        lam = kw.pop("lambdas", (0.5, 0.5))
        return synthetic(18.0, 8, 8, np.stack([qa, np.zeros(8)], 1), lam, seed, **kw)
    kw.setdefault("any_atom", True)
    if cfg == 2:
        qa = neutral_charges(qrng, 50, 0.4)
        lam = kw.pop("lambdas", (0.5, 0.5))
        return synthetic(30.0, 2000, 50, np.stack([qa, np.zeros(50)], 1), lam, seed, **kw)
    if cfg == 4:
        qs = np.stack([neutral_charges(qrng, 30, 0.5) for _ in range(4)], 1)
        lam = kw.pop("lambdas", (0.25, 0.25, 0.25, 0.25))
        off = [(i + 1, j + 1, 1, 2, 20.0, 0.0) for i in range(4) for j in range(i + 1, 4)]
        return synthetic(35.0, 3000, 30, qs, lam, seed, offdiag=off, **kw)
    if cfg == 5:
        qa = neutral_charges(qrng, 60, 0.4)
        lam = kw.pop("lambdas", (0.5, 0.5))
        return synthetic(40.0, 4000, 60, np.stack([qa, np.zeros(60)], 1), lam, seed, **kw)
    raise ValueError(f"unknown config {cfg}")


def lambda_batch_member(i: int, nwindows: int = 21, replicas: int = 11, rank: int = 0, **kw) -> System:
    """Trajectory i of lambda_batch(nwindows, replicas, rank), built alone.
    Different ranks (GPUs of a multi-GPU run) get the same recipe with their
    own seeds: independent replicas."""
    if not 0 <= i < nwindows + replicas:
        raise IndexError(i)
    if i < nwindows:
        la = 1.0 - i / (nwindows - 1) if nwindows > 1 else 0.5
        return config(1, window=i, replica=rank, lambdas=(la, 1.0 - la), **kw)
    r = i - nwindows
    R = (20.0, 25.0, 30.0)[r % 3]
    qa = neutral_charges(np.random.default_rng(1000), 8, 0.4)
    ns = 500 + int(round(1500 * r / max(replicas - 1, 1)))
    ns = min(ns, {20.0: 800, 25.0: 1500, 30.0: 2000}[R])
    kw.setdefault("any_atom", True)
    return synthetic(R, ns, 8, np.stack([qa, np.zeros(8)], 1), (0.5, 0.5), 3000 + 100 * r + 50000 * rank, **kw)


def lambda_batch(nwindows: int = 21, replicas: int = 11, rank: int = 0, **kw) -> list[System]:
    """The lambda-window batch: nwindows windows (lambda_A from 1 to 0) of the
    18 A droplet plus uneven replicas (spheres of 20/25/30 A with 500- to
    2,000-atom solutes, 8 Q atoms at lambda 0.5)."""
    return [lambda_batch_member(i, nwindows, replicas, rank, **kw) for i in range(nwindows + replicas)]
