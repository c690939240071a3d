"""Readers for Q's topology (.top), FEP (.fep) and MD input (.inp) files.

These are the host-side inputs that qdyn's Fortran master reads before md_run
(src/qdyn.f90:110-124).  The readers return plain dicts of numpy arrays in the
reference's own (1-based) numbering; :mod:`qsource_gb300.system` turns them into
the engine's 0-based descriptor.

Format references:
  .top  topo_read, src/topo.f90:515-1076 (writer topo_save :1077-1380)
  .fep  qatom_load_atoms / qatom_load_fep, src/qatom.f90:301-2035
  .inp  initialize, src/md.f90:4453-5358 (INI sections, src/prmfile.f90)
"""
from __future__ import annotations

import re
from typing import Callable

import numpy as np

MAX_NBR_RANGE = 25  # src/topo.f90:27


class _Records:
    """Line cursor that mimics Fortran list-directed and formatted reads."""

    def __init__(self, text: str):
        self.lines = text.splitlines()
        self.pos = 0

    def line(self) -> str:
        if self.pos >= len(self.lines):
            raise ValueError("unexpected end of file")
        s = self.lines[self.pos]
        self.pos += 1
        return s

    def skip(self, n: int = 1) -> None:
        for _ in range(n):
            self.line()

    def values(self, n: int, conv: Callable[[str], object]) -> list:
        """List-directed read of n items: starts at the next record, spans
        records, and drops the rest of the last record."""
        out: list = []
        while len(out) < n:
            for tok in self.line().replace(",", " ").split():
                if len(out) == n:
                    break
                out.append(conv(tok))
        return out

    def lead_ints(self, maxn: int) -> list[int]:
        """Leading integers of the next record, up to the first non-integer."""
        out = []
        for tok in self.line().split():
            if len(out) == maxn or not re.fullmatch(r"[+-]?\d+", tok):
                break
            out.append(int(tok))
        return out

    def digits(self, n: int, width: int = 80) -> str:
        """Formatted (80i1)/(80l1) read of n one-character fields."""
        out = []
        while len(out) < n:
            rec = self.line().ljust(width)[:width]
            out.extend(rec[: n - len(out)])
        return "".join(out)


def _f(tok: str) -> float:
    return float(tok.replace("D", "E").replace("d", "e"))


def read_top(text: str) -> dict:
    """Parse a Q topology; returns arrays in 1-based atom numbering."""
    r = _Records(text)
    t: dict = {}
    title = r.line().strip()
    t["version"] = 2.0
    if title == "Q topology file":
        while True:
            ln = r.line()
            key = ln.split()[0].upper() if ln.split() else ""
            rest = ln[len(ln.split()[0]):].strip() if ln.split() else ""
            if key == "VERSION":
                t["version"] = float(rest.split()[0])
            elif key == "FF_TYPE":
                t["ff_type"] = int(rest.split()[0])
            elif key == "END":
                break
    t.setdefault("ff_type", 1)
    head = r.lead_ints(3)
    nat = head[0]
    nat_solute = head[1] if len(head) > 1 else nat
    solv_atom = head[2] if len(head) > 2 else 3
    t["natom"], t["nat_solute"], t["solv_atom"] = nat, nat_solute, solv_atom
    t["xtop"] = np.array(r.values(3 * nat, _f), dtype=np.float64)
    r.skip()
    t["iac"] = np.array(r.values(nat, int), dtype=np.int32)
    # bonds
    h = r.lead_ints(2)
    nb = h[0]; t["nbonds_solute"] = h[1] if len(h) > 1 else nb
    t["bnd"] = np.array(r.values(3 * nb, int), dtype=np.int32).reshape(nb, 3)
    nbc = r.values(1, int)[0]
    lib = []
    for _ in range(nbc):
        tok = r.line().split()
        lib.append((_f(tok[1]), _f(tok[2])))
    t["bondlib"] = np.array(lib, dtype=np.float64).reshape(nbc, 2)
    # angles
    h = r.lead_ints(2)
    na = h[0]; t["nangles_solute"] = h[1] if len(h) > 1 else na
    t["ang"] = np.array(r.values(4 * na, int), dtype=np.int32).reshape(na, 4)
    nac = r.values(1, int)[0]
    lib = []
    for _ in range(nac):
        tok = r.line().split()
        vals = []
        for x in tok[1:5]:
            try:
                vals.append(_f(x))
            except ValueError:
                break
        vals += [0.0] * (4 - len(vals))
        lib.append(vals)
    t["anglib"] = np.array(lib, dtype=np.float64).reshape(nac, 4)
    # torsions
    h = r.lead_ints(2)
    nt = h[0]; t["ntors_solute"] = h[1] if len(h) > 1 else nt
    t["tor"] = np.array(r.values(5 * nt, int), dtype=np.int32).reshape(nt, 5)
    ntc = r.values(1, int)[0]
    lib = []
    for _ in range(ntc):
        v = r.values(5, _f)
        lib.append(v[1:5])
    t["torlib"] = np.array(lib, dtype=np.float64).reshape(ntc, 4)
    # impropers
    h = r.lead_ints(2)
    ni = h[0]; t["nimps_solute"] = h[1] if len(h) > 1 else ni
    t["imp"] = np.array(r.values(5 * ni, int), dtype=np.int32).reshape(ni, 5)
    h = r.lead_ints(2)
    nic = h[0]; t["imp_type"] = h[1] if len(h) > 1 else 1
    lib = []
    for _ in range(nic):
        v = r.values(3, _f)
        lib.append(v[1:3])
    t["implib"] = np.array(lib, dtype=np.float64).reshape(nic, 2)
    # charges
    r.skip()
    t["crg"] = np.array(r.values(nat, _f), dtype=np.float64)
    # charge groups
    h = r.lead_ints(3)
    ncgp = h[0]
    t["ncgp_solute"] = h[1] if len(h) > 1 else ncgp
    t["iuse_switch_atom"] = h[2] if len(h) > 2 else 1
    first, last, sw, atoms = [], [], [], []
    for _ in range(ncgp):
        n, isw = r.values(2, int)
        first.append(len(atoms) + 1)
        atoms.extend(r.values(n, int))
        last.append(len(atoms))
        sw.append(isw)
    t["cgp_first"] = np.array(first, dtype=np.int32)
    t["cgp_last"] = np.array(last, dtype=np.int32)
    t["cgp_switch"] = np.array(sw, dtype=np.int32)
    t["cgpatom"] = np.array(atoms, dtype=np.int32)
    # atom types
    natyps = r.values(1, int)[0]
    t["ivdw_rule"] = r.values(1, int)[0]
    ln = r.line().split()
    t["el14_scale"] = _f(ln[0])
    try:
        cc = _f(ln[1])
        t["coulomb_constant"] = cc if cc > 0 else 332.0
    except (IndexError, ValueError):
        t["coulomb_constant"] = 332.0
    r.skip()
    t["mass"] = np.array(r.values(natyps, _f), dtype=np.float64)
    av = np.zeros((natyps, 3)); bv = np.zeros((natyps, 3))
    for j in range(3):
        r.skip()
        av[:, j] = r.values(natyps, _f)
        r.skip()
        bv[:, j] = r.values(natyps, _f)
    t["avdw"], t["bvdw"] = av, bv
    nlj2 = r.values(1, int)[0]
    t["lj2"] = np.array([r.values(2, int) for _ in range(nlj2)], dtype=np.int32).reshape(nlj2, 2)
    # 1-4 neighbours and exclusions (bitmaps over max_nbr_range + long lists)
    r.values(1, int)
    bits14 = r.digits(MAX_NBR_RANGE * nat_solute) if nat_solute > 0 else ""
    n14l = r.values(1, int)[0]
    t["list14long"] = np.array([r.values(2, int) for _ in range(n14l)], dtype=np.int32).reshape(n14l, 2)
    r.values(1, int)
    bitsex = r.digits(MAX_NBR_RANGE * nat_solute) if nat_solute > 0 else ""
    nexl = r.values(1, int)[0]
    t["listexlong"] = np.array([r.values(2, int) for _ in range(nexl)], dtype=np.int32).reshape(nexl, 2)
    t["list14"] = _bitmap_pairs(bits14, nat_solute)
    t["listex"] = _bitmap_pairs(bitsex, nat_solute)
    # residues, molecules, type names
    ln = r.line()
    if ln.strip() == "":
        ln = r.line()
    nres = int(ln.split()[0])
    # "nres nres_solute" (the second number only when some residues are solvent)
    p2 = ln.split()
    t["nres"] = nres
    t["nres_solute"] = int(p2[1]) if len(p2) > 1 and re.fullmatch(r"\d+", p2[1]) else nres
    r.values(nres, int)
    r.skip()
    r.skip((nres + 15) // 16)
    nmol = r.values(1, int)[0]
    t["istart_mol"] = np.array(r.values(nmol, int), dtype=np.int32)
    r.skip()
    r.skip((natyps + 7) // 8)
    r.skip()
    r.skip((natyps + 12) // 13)
    t["solvent_type"] = r.values(1, int)[0]
    ln = r.line().split()
    t["use_pbc"] = ln[0] == "PBC"
    if t["use_pbc"]:
        # periodic box (src/topo.f90:1023-1031): box edges and centre; no
        # excluded atoms and no sphere
        t["boxlength"] = np.array(r.values(3, _f))
        t["boxcentre"] = np.array(r.values(3, _f))
        t["rexcl_o"], t["rwat"] = 0.0, 0.0
        t["xpcent"] = t["boxcentre"].copy()
        t["xwcent"] = t["boxcentre"].copy()
        t["nexats"], t["nexwat"] = 0, 0
        t["excl"] = np.zeros(nat, dtype=np.uint8)
        return t
    if t["version"] < 5.01:
        t["rexcl_o"], t["rexcl_i_top"], t["rwat"] = _f(ln[0]), _f(ln[1]), _f(ln[2])
    else:
        t["rexcl_o"], t["rwat"] = _f(ln[0]), _f(ln[1])
    t["xpcent"] = np.array(r.values(3, _f))
    t["xwcent"] = np.array(r.values(3, _f))
    t["nexats"], t["nexwat"] = r.values(2, int)
    flags = r.digits(nat)
    t["excl"] = np.array([c in "Tt" for c in flags], dtype=np.uint8)
    return t


def _bitmap_pairs(bits: str, nat_solute: int) -> np.ndarray:
    """(i, i+k) pairs (1-based) of a list14/listex bitmap read as
    ((temp(k, j), k=1..25), j=1..nat_solute), src/topo.f90:915-924."""
    out = []
    for j in range(nat_solute):
        row = bits[j * MAX_NBR_RANGE:(j + 1) * MAX_NBR_RANGE]
        for k, c in enumerate(row):
            if c == "1":
                out.append((j + 1, j + 1 + k + 1))
    return np.array(out, dtype=np.int32).reshape(-1, 2)


# --------------------------------------------------------------- INI files
def _sections(text: str) -> dict[str, list[str]]:
    """INI-like [section] / line map of prmfile.f90 (comments after ! or #)."""
    secs: dict[str, list[str]] = {}
    cur = None
    for raw in text.splitlines():
        ln = re.split(r"[!#]", raw, maxsplit=1)[0].strip()
        if not ln:
            continue
        m = re.fullmatch(r"\[(.+?)\]", ln)
        if m:
            cur = m.group(1).strip().lower()
            secs.setdefault(cur, [])
            continue
        if cur is not None:
            secs[cur].append(ln)
    return secs


def read_inp(text: str) -> dict:
    """The subset of the qdyn .inp file that the hot path needs."""
    secs = _sections(text)

    def kv(sec: str) -> dict[str, str]:
        out = {}
        for ln in secs.get(sec, []):
            p = ln.split(None, 1)
            out[p[0].lower()] = p[1].strip() if len(p) > 1 else ""
        return out

    md, cut, sph, solv, inter, files = (kv("md"), kv("cut-offs"), kv("sphere"), kv("solvent") or kv("water"),
                                        kv("intervals"), kv("files"))

    def onoff(s, default):
        if s is None:
            return default
        return s.strip().lower() in ("on", "true", ".true.", "1", "yes")

    lam = []
    for ln in secs.get("lambdas", []):
        lam.extend(float(x) for x in ln.split())
    # [sequence_restraints]: atom_i atom_j fc H-flag to_centre (initialize,
    # src/md.f90:5215-5233; to_centre defaults to 0)
    rstseq = []
    for ln in secs.get("sequence_restraints", []):
        t = ln.split()
        if len(t) >= 3:
            rstseq.append((int(t[0]), int(t[1]), float(t[2]), int(t[3]) if len(t) > 3 else 0,
                           int(t[4]) if len(t) > 4 else 0))

    # [atom_restraints] / [distance_restraints] / [angle_restraints] /
    # [wall_restraints] (initialize, src/md.f90:5234-5358); the residue:atom
    # form of distance restraints is not read
    def rows(sec, nint_lead, nflt, ntail_int):
        out = []
        for ln in secs.get(sec, []):
            t = ln.split()
            if any(":" in x for x in t):
                raise ValueError(f"[{sec}]: residue:atom references are not supported")
            out.append([int(x) for x in t[:nint_lead]] + [float(x) for x in t[nint_lead:nint_lead + nflt]] +
                       [int(x) for x in t[nint_lead + nflt:nint_lead + nflt + ntail_int]])
        return out

    rst_pos = rows("atom_restraints", 1, 6, 1)
    rst_dist = rows("distance_restraints", 2, 3, 1)
    rst_angl = rows("angle_restraints", 3, 2, 1)
    rst_wall = rows("wall_restraints", 2, 4, 1)

    def real(d, key, default=None):
        return float(d[key]) if key in d else default

    wpol = onoff(solv.get("polarisation"), True)
    # [PBC] (initialize, src/md.f90:4514-4590); constant pressure is not supported
    pbc = kv("pbc")
    return {
        "pbc": "pbc" in secs,
        "put_solute_back_in_box": onoff(pbc.get("put_solute_back_in_box"), False),
        "put_solvent_back_in_box": onoff(pbc.get("put_solvent_back_in_box"), False),
        "rigid_box_centre": onoff(pbc.get("rigid_box_centre"), False),
        "constant_pressure": onoff(pbc.get("constant_pressure"), False),
        "steps": int(md.get("steps", 0)),
        "stepsize": float(md.get("stepsize", 1.0)),
        "temperature": float(md.get("temperature", 300.0)),
        "bath_coupling": float(md.get("bath_coupling", 100.0)),
        "thermostat": md.get("thermostat", "berendsen"),
        "integrator": md.get("integrator", "leap-frog"),
        "separate_scaling": onoff(md.get("separate_scaling"), True),
        "random_seed": int(md.get("random_seed", 1)),
        "initial_temperature": float(md["initial_temperature"]) if "initial_temperature" in md else None,
        "shake_solvent": onoff(md.get("shake_solvent"), True),
        "shake_solute": onoff(md.get("shake_solute"), False),
        "shake_hydrogens": onoff(md.get("shake_hydrogens"), False),
        "lrf": onoff(md.get("lrf"), True),
        "Rcpp": float(cut.get("solute_solute", 10.0)),
        "Rcww": float(cut.get("solvent_solvent", 10.0)),
        "Rcpw": float(cut.get("solute_solvent", 10.0)),
        "Rcq": float(cut.get("q_atom", 99.0)),
        "RcLRF": float(cut.get("lrf", 99.0)),
        "shell_radius": float(sph["shell_radius"]) if "shell_radius" in sph else None,
        "shell_force": float(sph.get("shell_force", 10.0)),
        "excluded_force": float(sph.get("excluded_force", 200.0)),
        "solvent_radius": float(solv["radius"]) if "radius" in solv else None,
        "radial_force": float(solv["radial_force"]) if "radial_force" in solv else -1.0,
        "polarisation": wpol,
        "charge_correction": onoff(solv.get("charge_correction"), wpol),
        "polarisation_force": real(solv, "polarisation_force", -1.0),
        "excluded_freeze": onoff(sph.get("excluded_freeze"), False),
        "sequence_restraints": rstseq,
        "atom_restraints": rst_pos, "distance_restraints": rst_dist, "angle_restraints": rst_angl,
        "wall_restraints": rst_wall,
        "langevin_friction": real(md, "langevin_friction"),
        "langevin_random": onoff(md.get("langevin_random"), False),
        "nhchains": int(md["nhchains"]) if "nhchains" in md else 10,
        "nose_hoover_mass": real(md, "nose-hoover_mass"),
        "morse_depth": float(solv.get("morse_depth", -1.0)),
        "morse_width": float(solv.get("morse_width", -1.0)),
        "non_bond": int(inter.get("non_bond", 10)),
        "lambdas": lam,
        "topology": files.get("topology"),
        "fep": files.get("fep"),
        "unsupported": [s for s in secs if s in ("group_contribution",)],
    }


def read_fep(text: str) -> dict:
    """The [FEP]/[atoms]/charges/types/bonded sections of a Q FEP file."""
    secs = _sections(text)
    fep: dict = {}
    kv = {ln.split(None, 1)[0].lower(): ln.split(None, 1)[1] for ln in secs.get("fep", []) if len(ln.split()) > 1}
    fep["nstates"] = int(kv.get("states", 1))
    offset = int(kv.get("offset", 0))
    # [PBC] switching_atom: the atom the Q-atom lists are centred on in a
    # periodic box (qatom_load_fep, src/qatom.f90:672-687)
    pb = {ln.split(None, 1)[0].lower(): ln.split(None, 1)[1] for ln in secs.get("pbc", []) if len(ln.split()) > 1}
    fep["qswitch"] = int(pb["switching_atom"]) + offset if "switching_atom" in pb else None
    if "offset_name" in kv or "offset_residue" in kv:
        raise ValueError("[FEP] offset_name/offset_residue are not supported")
    atoms = {}
    for ln in secs.get("atoms", []):
        p = ln.split()
        atoms[int(p[0])] = int(p[1]) + offset
    nq = max(atoms) if atoms else 0
    fep["iqseq"] = np.array([atoms[i] for i in range(1, nq + 1)], dtype=np.int32)
    S = fep["nstates"]

    def rows(sec, nint, nflt=0):
        out = []
        for ln in secs.get(sec, []):
            p = ln.split()
            out.append([int(x) for x in p[:nint]] + [_f(x) for x in p[nint:nint + nflt]])
        return out

    fep["change_charges"] = [(int(p[0]), [_f(x) for x in p[1:1 + S]]) for p in map(str.split, secs.get("change_charges", []))]
    fep["atom_types"] = []
    for ln in secs.get("atom_types", []):
        p = ln.split()
        fep["atom_types"].append((p[0], [_f(x) for x in p[1:7]], _f(p[7])))
    fep["change_atoms"] = [(int(p[0]), p[1:1 + S]) for p in map(str.split, secs.get("change_atoms", []))]
    fep["soft_pairs"] = rows("soft_pairs", 2)
    fep["el_scale"] = [(int(p[0]), int(p[1]), [_f(x) for x in p[2:2 + S]]) for p in map(str.split, secs.get("el_scale", []))]
    fep["excluded_pairs"] = [(int(p[0]) + offset, int(p[1]) + offset, [int(x) for x in p[2:2 + S]])
                             for p in map(str.split, secs.get("excluded_pairs", []))]
    # bond types: Morse "j Dmz amz r0" when four numbers parse, else harmonic "j fk r0"
    # (qatom_load_fep, src/qatom.f90:838-868)
    btypes = {}
    for ln in secs.get("bond_types", []):
        p = ln.split()
        nums = []
        for x in p[1:4]:
            try:
                nums.append(_f(x))
            except ValueError:
                break
        if len(nums) == 3:
            btypes[int(p[0])] = (nums[0], nums[1], nums[2], 0.0)
        else:
            btypes[int(p[0])] = (0.0, 0.0, nums[1], nums[0])
    fep["bond_types"] = btypes
    fep["change_bonds"] = [(int(p[0]) + offset, int(p[1]) + offset, [int(x) for x in p[2:2 + S]])
                           for p in map(str.split, secs.get("change_bonds", []))]
    atypes = {}
    for ln in secs.get("angle_types", []):
        p = ln.split()
        nums = []
        for x in p[1:5]:
            try:
                nums.append(_f(x))
            except ValueError:
                break
        nums += [0.0] * (4 - len(nums))
        atypes[int(p[0])] = tuple(nums)
    fep["angle_types"] = atypes
    fep["change_angles"] = [(tuple(int(x) + offset for x in p[0:3]), [int(x) for x in p[3:3 + S]])
                            for p in map(str.split, secs.get("change_angles", []))]
    fep["torsion_types"] = {int(p[0]): (_f(p[1]), _f(p[2]), _f(p[3])) for p in map(str.split, secs.get("torsion_types", []))}
    fep["change_torsions"] = [(tuple(int(x) + offset for x in p[0:4]), [int(x) for x in p[4:4 + S]])
                              for p in map(str.split, secs.get("change_torsions", []))]
    fep["improper_types"] = {int(p[0]): (_f(p[1]), _f(p[2])) for p in map(str.split, secs.get("improper_types", []))}
    fep["change_impropers"] = [(tuple(int(x) + offset for x in p[0:4]), [int(x) for x in p[4:4 + S]])
                               for p in map(str.split, secs.get("change_impropers", []))]
    fep["off_diagonals"] = [(int(p[0]), int(p[1]), int(p[2]), int(p[3]), _f(p[4]), _f(p[5]))
                            for p in map(str.split, secs.get("off_diagonals", []))]
    unsupported = [s for s in ("angle_couplings", "torsion_couplings", "improper_couplings", "shake_constraints",
                               "softcore", "monitor_groups", "monitor_group_pairs") if secs.get(s)]
    fep["unsupported"] = unsupported
    return fep
