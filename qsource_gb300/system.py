"""Host-side system set-up: the qdyn start-up sequence that precedes md_run.

``System`` holds the flat 0-based arrays of one trajectory and turns them into
the ``qgpu_system_desc`` of include/qgpu.h.  It is built either from Q's own
input files (``System.from_files``: topology, prep_coord, get_fep, prep_sim,
init_shake, make_nbqqlist, shrink_topology, src/qdyn.f90:110-124) or from the
seeded synthetic water-sphere generator in :mod:`qsource_gb300.synth`.
"""
from __future__ import annotations

import ctypes as C
import math
from collections import deque

import numpy as np

from . import qtop
from .abi import MAX_STATES, SystemDesc, ptr

BOLTZ = 0.001986                 # src/md.f90:54
TIME_UNIT = 0.020462             # fs -> internal time (src/md.f90:4623)
DEG2RAD = math.pi / 180.0


class System:
    """Arrays of one trajectory in the engine's 0-based layout."""

    def __init__(self, **kw):
        self.__dict__.update(kw)
        self._keep: list = []

    # ---------------------------------------------------------------- desc
    def desc(self) -> SystemDesc:
        """Fill a qgpu_system_desc.  The arrays it points to are held by the
        returned descriptor (and by self._keep until the next call), so a
        descriptor stays valid however many others are made later."""
        d = SystemDesc()
        keep: list = []
        self._keep = keep
        d._keep = keep

        def arr(a, dt):
            if a is None:
                return None
            b = np.ascontiguousarray(a, dtype=dt)
            if b.size == 0:
                b = np.zeros(1, dtype=dt)
            keep.append(b)
            return ptr(b)

        S = self.nstates
        d.natom, d.nat_solute, d.solv_atom, d.nwat = self.natom, self.nat_solute, 3, self.nwat
        d.natyps, d.ncgp, d.ncgp_solute = self.natyps, len(self.cgp_first), self.ncgp_solute
        d.nqat, d.nstates = self.nqat, S
        d.x, d.v, d.xtop = arr(self.x, np.float64), arr(self.v, np.float64), arr(self.xtop, np.float64)
        d.crg, d.iac = arr(self.crg, np.float64), arr(self.iac, np.int32)
        d.excl, d.shell, d.iqatom = arr(self.excl, np.uint8), arr(self.shell, np.uint8), arr(self.iqatom, np.int32)
        d.mass, d.avdw, d.bvdw = arr(self.mass, np.float64), arr(self.avdw, np.float64), arr(self.bvdw, np.float64)
        d.ljcod = arr(self.ljcod, np.int8)
        d.el14_scale, d.ivdw_rule, d.ff_type = self.el14_scale, int(getattr(self, "ivdw_rule", 1)), self.ff_type
        for k in range(3):
            d.chg_solv[k] = self.chg_solv[k]
        for k in range(6):
            d.aLJ_solv[k] = self.aLJ_solv.ravel()[k]
            d.bLJ_solv[k] = self.bLJ_solv.ravel()[k]
        d.cgp_first, d.cgp_last = arr(self.cgp_first, np.int32), arr(self.cgp_last, np.int32)
        d.cgp_switch, d.cgpatom = arr(self.cgp_switch, np.int32), arr(self.cgpatom, np.int32)
        d.nexcl, d.excl_pairs = len(self.excl_pairs), arr(self.excl_pairs, np.int32)
        d.n14, d.pairs14 = len(self.pairs14), arr(self.pairs14, np.int32)
        d.iqseq, d.qcrg = arr(self.iqseq, np.int32), arr(self.qcrg, np.float64)
        d.qvdw_flag, d.qiac, d.nqlib = int(self.qvdw_flag), arr(self.qiac, np.int32), len(self.qavdw)
        d.qavdw, d.qbvdw = arr(self.qavdw, np.float64), arr(self.qbvdw, np.float64)
        d.sc_lookup = arr(self.sc_lookup, np.float64)
        for s in range(S):
            d.lambda_[s] = self.lambdas[s]
        d.qp_skip = arr(self.qp_skip, np.uint8)
        d.nqp14, d.qp14_pairs = len(self.qp14_pairs), arr(self.qp14_pairs, np.int32)
        for s in range(S):
            d.nbqq_count[s] = self.nbqq_count[s]
        d.nbqq_iq, d.nbqq_j = arr(self.nbqq["iq"], np.int32), arr(self.nbqq["j"], np.int32)
        d.nbqq_jq, d.nbqq_ljcod = arr(self.nbqq["jq"], np.int32), arr(self.nbqq["lj"], np.int8)
        d.nbqq_elscale = arr(self.nbqq["els"], np.float64)
        d.nqbond, d.qbnd = len(self.qbnd), arr(self.qbnd, np.int32)
        d.nqbcod, d.qbondlib = len(self.qbondlib), arr(self.qbondlib, np.float64)
        d.nqangle, d.qang = len(self.qang), arr(self.qang, np.int32)
        d.nqacod, d.qanglib = len(self.qanglib), arr(self.qanglib, np.float64)
        d.nqtor, d.qtor = len(self.qtor), arr(self.qtor, np.int32)
        d.nqtcod, d.qtorlib = len(self.qtorlib), arr(self.qtorlib, np.float64)
        d.nqimp, d.qimp = len(self.qimp), arr(self.qimp, np.int32)
        d.nqicod, d.qimplib = len(self.qimplib), arr(self.qimplib, np.float64)
        d.nbonds, d.nbonds_solute, d.bnd = len(self.bnd), self.nbonds_solute, arr(self.bnd, np.int32)
        d.nbndcod, d.bondlib = len(self.bondlib), arr(self.bondlib, np.float64)
        d.nangles, d.nangles_solute, d.ang = len(self.ang), self.nangles_solute, arr(self.ang, np.int32)
        d.nangcod, d.anglib = len(self.anglib), arr(self.anglib, np.float64)
        d.ntors, d.ntors_solute, d.tor = len(self.tor), self.ntors_solute, arr(self.tor, np.int32)
        d.ntorcod, d.torlib = len(self.torlib), arr(self.torlib, np.float32)
        d.nimps, d.nimps_solute, d.imp = len(self.imp), self.nimps_solute, arr(self.imp, np.int32)
        d.nimpcod, d.implib = len(self.implib), arr(self.implib, np.float32)
        d.shake_molecules = len(self.shake_first) - 1
        d.shake_first, d.shake_i = arr(self.shake_first, np.int32), arr(self.shake_i, np.int32)
        d.shake_j, d.shake_dist2 = arr(self.shake_j, np.int32), arr(self.shake_dist2, np.float64)
        d.noffd = len(self.offd)
        offd = np.array(self.offd, dtype=np.float64).reshape(-1, 6)
        d.offd_ij = arr(offd[:, 0:2], np.int32)
        d.offd_kl = arr(offd[:, 2:4], np.int32)
        d.offd_Amu = arr(offd[:, 4:6], np.float64)
        for k in range(3):
            d.xpcent[k] = self.xpcent[k]
            d.xwcent[k] = self.xwcent[k]
        d.rexcl_o, d.rwat = self.rexcl_o, self.rwat
        d.fk_wsphere, d.Dwmz, d.awmz = self.fk_wsphere, self.Dwmz, self.awmz
        d.fk_pshell, d.fk_fix, d.wpol_restr = self.fk_pshell, self.fk_fix, int(self.wpol_restr)
        d.Rcpp, d.Rcww, d.Rcpw, d.Rcq, d.RcLRF = self.Rcpp, self.Rcww, self.Rcpw, self.Rcq, self.RcLRF
        d.use_LRF = int(self.use_LRF)
        d.dt, d.Temp0, d.tau_T = self.dt, self.Temp0, self.tau_T
        d.separate_scaling, d.NBcycle = int(self.separate_scaling), self.NBcycle
        for k in ("Ndegf", "Ndegfree", "Ndegf_solvent", "Ndegfree_solvent", "Ndegf_solute", "Ndegfree_solute"):
            setattr(d, k, int(getattr(self, k)))
        d.detail_temps = int(self.detail_temps)
        d.any_atom_lists = int(getattr(self, "any_atom_lists", 0))
        g = lambda k, dflt: getattr(self, k, dflt)
        rij = np.asarray(g("rstseq_ij", np.zeros((0, 2), np.int32)), dtype=np.int32).reshape(-1, 2)
        d.nrstr_seq = len(rij)
        d.rstseq_ij = arr(rij, np.int32)
        d.rstseq_fk = arr(np.asarray(g("rstseq_fk", np.zeros(0))), np.float64)
        d.rstseq_flags = arr(np.asarray(g("rstseq_flags", np.zeros((0, 2), np.int32))).reshape(-1, 2), np.int32)
        heavy = g("heavy", None)
        if heavy is None:
            heavy = (np.asarray(self.mass)[np.asarray(self.iac)] >= 4.0).astype(np.uint8)
        d.heavy = arr(np.asarray(heavy), np.uint8)
        d.excluded_freeze = int(g("excluded_freeze", 0))
        wsh = np.asarray(g("wshell", np.zeros((0, 4))), dtype=np.float64).reshape(-1, 4)
        d.fkwpol = float(g("fkwpol", 20.0))
        d.nwpolr_shell = len(wsh)
        d.wshell_rout = arr(wsh[:, 0], np.float64)
        d.wshell_dr = arr(wsh[:, 1], np.float64)
        d.wshell_cstb = arr(wsh[:, 2], np.float64)
        d.wshell_theta_corr = arr(wsh[:, 3], np.float64)
        d.itdis_update = int(g("itdis_update", 100))
        d.thermostat = int(g("thermostat", 0))
        d.integrator = int(g("integrator", 0))
        d.friction = float(g("friction", 1.0 / self.tau_T))
        d.langevin_gauss = int(g("langevin_gauss", 0))
        d.rand_state = int(g("rand_state", 1))
        d.nhchains = int(g("nhchains", 10))
        d.nhq = float(g("nhq", 0.001986 * self.Temp0 / (self.tau_T * self.tau_T)))
        d.use_pbc = int(g("use_pbc", 0))
        for k in range(3):
            d.boxlength[k] = float(np.asarray(g("boxlength", np.zeros(3)))[k])
            d.boxcentre[k] = float(np.asarray(g("boxcentre", np.zeros(3)))[k])
        d.qswitch = int(g("qswitch", -1))
        d.put_solute_back = int(g("put_solute_back", 0))
        d.put_solvent_back = int(g("put_solvent_back", 0))
        d.rigid_box_centre = int(g("rigid_box_centre", 0))
        im = np.asarray(g("istart_mol", np.zeros(0, np.int32)), dtype=np.int32)
        d.nmol = len(im)
        d.istart_mol = arr(im, np.int32)
        d.nsolute_mol = int(g("nsolute_mol", 0))
        for name, ni, nf in (("rstpos", 2, 6), ("rstdis", 3, 3), ("rstang", 4, 2), ("rstwal", 3, 4)):
            ia = np.asarray(g(f"{name}_i", np.zeros((0, ni), np.int32)), dtype=np.int32).reshape(-1, ni)
            fa = np.asarray(g(f"{name}_{'x' if name == 'rstpos' else 'p'}", np.zeros((0, nf))),
                            dtype=np.float64).reshape(-1, nf)
            setattr(d, {"rstpos": "nrstr_pos", "rstdis": "nrstr_dist", "rstang": "nrstr_angl",
                        "rstwal": "nrstr_wall"}[name], len(ia))
            setattr(d, f"{name}_i", arr(ia, np.int32))
            setattr(d, f"{name}_{'x' if name == 'rstpos' else 'p'}", arr(fa, np.float64))
        return d

    @property
    def nwat(self) -> int:
        return (self.natom - self.nat_solute) // 3

    # ------------------------------------------------------------ fixtures
    def save_npz(self, path: str) -> None:
        """Store every field (arrays, scalars, lists, the nbqq dict) in one npz."""
        out = {}
        for k, v in self.__dict__.items():
            if k.startswith("_"):
                continue
            if isinstance(v, dict):
                for kk, vv in v.items():
                    out[f"dict:{k}:{kk}"] = np.asarray(vv)
            elif isinstance(v, list) and v and isinstance(v[0], tuple):
                out[f"tuples:{k}"] = np.asarray(v, dtype=np.float64).reshape(len(v), -1)
            elif isinstance(v, list):
                out[f"list:{k}"] = np.asarray(v)
            elif v is None:
                out[f"none:{k}"] = np.zeros(0)
            else:
                out[f"val:{k}"] = np.asarray(v)
        np.savez_compressed(path, **out)

    @classmethod
    def load_npz(cls, path: str) -> "System":
        kw: dict = {}
        with np.load(path) as z:
            for key in z.files:
                kind, _, name = key.partition(":")
                a = z[key]
                if kind == "dict":
                    d, _, sub = name.partition(":")
                    kw.setdefault(d, {})[sub] = a
                elif kind == "tuples":
                    kw[name] = [tuple(r) for r in a.tolist()]
                elif kind == "list":
                    kw[name] = a.tolist()
                elif kind == "none":
                    kw[name] = None
                else:
                    kw[name] = a if a.ndim else a.item()
        for k in ("offd",):
            kw.setdefault(k, [])
        kw["offd"] = [tuple(int(x) if i < 4 else x for i, x in enumerate(r)) for r in kw["offd"]]
        return cls(**kw)

    # ----------------------------------------------------------- builders
    @classmethod
    def from_files(cls, top_text: str, fep_text: str | None, inp_text: str) -> "System":
        return build(qtop.read_top(top_text), qtop.read_fep(fep_text) if fep_text else None, qtop.read_inp(inp_text))


# --------------------------------------------------------------------------
def build(top: dict, fep: dict | None, inp: dict) -> System:
    """qdyn start-up on parsed inputs -> System (0-based)."""
    if top["solv_atom"] != 3 or top["solvent_type"] != 0:
        raise ValueError("only 3-site SPC-type solvent is supported (solvent_type 0)")
    if top["ivdw_rule"] not in (1, 2):
        raise ValueError(f"unknown combination rule ivdw_rule {top['ivdw_rule']} (1 geometric, 2 arithmetic)")
    if inp["unsupported"]:
        raise ValueError(f"unsupported input sections: {inp['unsupported']}")
    natom, nsol = top["natom"], top["nat_solute"]
    # periodic box: the topology's boundary and the input's [PBC] must agree
    # (src/md.f90:17869-17872)
    use_pbc = bool(top.get("use_pbc", False))
    if use_pbc != bool(inp.get("pbc", False)):
        raise ValueError("the boundary of the topology (sphere / PBC) and of the input must match")
    if use_pbc and inp.get("constant_pressure"):
        raise ValueError("[PBC] constant_pressure is not supported")
    natyps = len(top["mass"])
    cc = top["coulomb_constant"]
    sq = math.sqrt(cc)
    iac = top["iac"] - 1
    ljcod = np.ones((natyps, natyps), dtype=np.int8)
    for a, b in top["lj2"]:
        ljcod[a - 1, b - 1] = ljcod[b - 1, a - 1] = 2
    crg = top["crg"] * sq
    avdw, bvdw, mass = top["avdw"], top["bvdw"], top["mass"]
    heavy = mass[iac] >= 4.0
    excl = top["excl"].astype(np.uint8)
    xtop = top["xtop"].copy()
    cgp_first, cgp_last = top["cgp_first"] - 1, top["cgp_last"] - 1
    cgp_switch, cgpatom = top["cgp_switch"] - 1, top["cgpatom"] - 1
    ncgp_solute = top["ncgp_solute"]
    # --- sphere set-up (initialize [sphere]/[solvent], prep_coord make_shell, wat_sphere)
    rexcl_o = top["rexcl_o"]
    rexcl_i = inp["shell_radius"] if inp["shell_radius"] is not None else 0.85
    if rexcl_i <= 1.0:
        rexcl_i *= rexcl_o
    shell = np.zeros(natom, dtype=np.uint8)
    xp = top["xpcent"]
    for g in range(0 if use_pbc else ncgp_solute):
        s = cgp_switch[g]
        if not excl[s] and heavy[s]:
            if np.sum((xtop[3 * s:3 * s + 3] - xp) ** 2) > rexcl_i ** 2:
                shell[cgpatom[cgp_first[g]:cgp_last[g] + 1]] = 1
    rwat = inp["solvent_radius"] if inp["solvent_radius"] else top["rwat"]
    fk_wsphere = inp["radial_force"] if inp["radial_force"] != -1 else 60.0
    Dwmz = inp["morse_depth"] if inp["morse_depth"] != -1 else 0.26 * math.exp(-0.19 * (rwat - 15.0)) + 0.74
    awmz = inp["morse_width"] if inp["morse_width"] != -1 else 0.2 / (1.0 + math.exp(0.4 * (rwat - 25.0))) + 0.3
    fk_fix = inp["excluded_force"] if inp["excluded_force"] > 0 else 200.0

    # --- bonded topology (working copies; codes stay 1-based, 0 = removed, -1 = shaken)
    bnd = top["bnd"].copy(); bnd[:, :2] -= 1
    ang = top["ang"].copy(); ang[:, :3] -= 1
    tor = top["tor"].copy(); tor[:, :4] -= 1
    imp = top["imp"].copy(); imp[:, :4] -= 1
    excl_set = set(tuple(sorted((a - 1, b - 1))) for a, b in top["listex"])
    excl_set |= set(tuple(sorted((a - 1, b - 1))) for a, b in top["listexlong"])
    p14_set = set(tuple(sorted((a - 1, b - 1))) for a, b in top["list14"])
    p14_set |= set(tuple(sorted((a - 1, b - 1))) for a, b in top["list14long"])

    # --- Q atoms (get_fep, src/md.f90:2884-3074)
    S = fep["nstates"] if fep else 1
    lam = list(inp["lambdas"]) if inp["lambdas"] else [1.0]
    if fep is not None and len(lam) != S:
        raise ValueError(f"[lambdas] gives {len(lam)} values for {S} states")
    iqseq = fep["iqseq"] - 1 if fep else np.zeros(0, dtype=np.int32)
    nq = len(iqseq)
    iqatom = -np.ones(natom, dtype=np.int32)
    iqatom[iqseq] = np.arange(nq)
    qcrg = np.repeat(top["crg"][iqseq][:, None], S, axis=1)
    qvdw_flag = False
    qiac = np.repeat(np.arange(nq)[:, None], S, axis=1)
    qavdw, qbvdw = avdw[iac[iqseq]].copy(), bvdw[iac[iqseq]].copy()
    qbnd = np.zeros((0, 2 + S), dtype=np.int32); qbondlib = np.zeros((0, 4))
    qang = np.zeros((0, 3 + S), dtype=np.int32); qanglib = np.zeros((0, 4))
    qtor = np.zeros((0, 4 + S), dtype=np.int32); qtorlib = np.zeros((0, 3))
    qimp = np.zeros((0, 4 + S), dtype=np.int32); qimplib = np.zeros((0, 2))
    offd = []
    soft_pairs, el_scale, exspec = [], [], []
    if fep is not None:
        if fep["unsupported"]:
            raise ValueError(f"unsupported FEP sections: {fep['unsupported']}")
        for iq, vals in fep["change_charges"]:
            qcrg[iq - 1, :] = vals[:S]
        if fep["atom_types"]:
            names = {t[0]: k for k, t in enumerate(fep["atom_types"])}
            qavdw = np.array([[t[1][0], t[1][2], t[1][4]] for t in fep["atom_types"]])
            qbvdw = np.array([[t[1][1], t[1][3], t[1][5]] for t in fep["atom_types"]])
        if fep["change_atoms"]:
            if len(fep["change_atoms"]) != nq:
                raise ValueError("[change_atoms] must list every Q atom")
            qvdw_flag = True
            for iq, tn in fep["change_atoms"]:
                qiac[iq - 1, :] = [names[n] for n in tn[:S]]
        soft_pairs = [(a - 1, b - 1) for a, b in fep["soft_pairs"]]
        el_scale = [(a - 1, b - 1, v) for a, b, v in fep["el_scale"]]
        exspec = [(a - 1, b - 1, f) for a, b, f in fep["excluded_pairs"]]
        btypes = fep["bond_types"]
        if btypes:
            nb = max(btypes)
            qbondlib = np.array([btypes.get(k, (0, 0, 0, 0)) for k in range(1, nb + 1)], dtype=np.float64)
        qbnd = np.array([[i - 1, j - 1] + c for i, j, c in fep["change_bonds"]], dtype=np.int32).reshape(-1, 2 + S)
        at = fep["angle_types"]
        if at:
            qanglib = np.array([at.get(k, (0, 0, 0, 0)) for k in range(1, max(at) + 1)], dtype=np.float64)
            qanglib[:, 1] *= DEG2RAD
        qang = np.array([[a - 1 for a in ijk] + c for ijk, c in fep["change_angles"]], dtype=np.int32).reshape(-1, 3 + S)
        tt = fep["torsion_types"]
        if tt:
            qtorlib = np.array([tt.get(k, (0, 0, 0)) for k in range(1, max(tt) + 1)], dtype=np.float64)
            qtorlib[:, 2] *= DEG2RAD
        qtor = np.array([[a - 1 for a in t] + c for t, c in fep["change_torsions"]], dtype=np.int32).reshape(-1, 4 + S)
        it = fep["improper_types"]
        if it:
            qimplib = np.array([it.get(k, (0, 0)) for k in range(1, max(it) + 1)], dtype=np.float64)
            qimplib[:, 1] *= DEG2RAD
        qimp = np.array([[a - 1 for a in t] + c for t, c in fep["change_impropers"]], dtype=np.int32).reshape(-1, 4 + S)
        offd = [(i - 1, j - 1, k - 1, l - 1, A, mu) for i, j, k, l, A, mu in fep["off_diagonals"]]
        # remove redefined classical terms (get_fep, src/md.f90:2928-3010)
        for b in range(len(bnd)):
            for q in qbnd:
                if {bnd[b, 0], bnd[b, 1]} == {q[0], q[1]}:
                    bnd[b, 2] = 0
        for a in range(len(ang)):
            for q in qang:
                if (ang[a, 0], ang[a, 1], ang[a, 2]) in ((q[0], q[1], q[2]), (q[2], q[1], q[0])):
                    ang[a, 3] = 0
        for t in range(len(tor)):
            for q in qtor:
                if tor[t, 4] != 0 and (tuple(tor[t, :4]) in (tuple(q[:4]), (q[3], q[2], q[1], q[0]))):
                    tor[t, 4] = 0
        for p in range(len(imp)):
            i, j, k, l = imp[p, :4]
            for q in qimp:
                qi, qj, qk, ql = q[:4]
                if top["ff_type"] == 3:
                    raise ValueError("CHARMM improper redefinition is not supported")
                if ((i, j, k, l) == (qi, qj, qk, ql) or (i, j, k, l) == (qk, qj, qi, ql) or
                        (i, j, k, l) == (qk, qj, ql, qi) or (i, j, k, l) == (ql, qj, qi, qk) or
                        (i, j, k, l) == (ql, qj, qk, qi)):
                    imp[p, 4] = 0
        # special exclusions between a Q and a non-Q atom in all states
        for i, j, f in exspec:
            if iqatom[i] < 0 or iqatom[j] < 0:
                if any(f[:S]):
                    if not all(f[:S]):
                        raise ValueError("invalid special exclusion data")
                    excl_set.add(tuple(sorted((i, j))))
    qcrg = qcrg * sq

    # --- init_shake (src/md.f90:4242-4426)
    istart = list(top["istart_mol"] - 1) + [natom]
    nmol = len(istart) - 1
    mols: list[list[tuple[int, int, float]]] = [[] for _ in range(nmol)]
    mol = -1
    exclshk = 0.0
    sh_solv, sh_solu, sh_h = inp["shake_solvent"], inp["shake_solute"], inp["shake_hydrogens"]
    for b in range(len(bnd)):
        ia, ja, cod = bnd[b]
        while ia >= istart[mol + 1]:
            mol += 1
        if cod == 0:
            continue
        if (sh_h and (not heavy[ia] or not heavy[ja])) or (sh_solu and ia < nsol) or (sh_solv and ia >= nsol):
            mols[mol].append((ia, ja, top["bondlib"][cod - 1, 1] ** 2))
            if excl[ia]:
                exclshk += 0.5
            if excl[ja]:
                exclshk += 0.5
            bnd[b, 2] = -1
    nwat = (natom - nsol) // 3
    solute_constraints = sum(len(m) for m in mols[:nmol - nwat])
    shake_mols = [m for m in mols if m]
    nconstr = sum(len(m) for m in shake_mols)
    for m in shake_mols:
        for ia, ja, _ in m:
            for a in range(len(ang)):
                if (ang[a, 0] == ia and ang[a, 2] == ja) or (ang[a, 0] == ja and ang[a, 2] == ia):
                    ang[a, 3] = 0
                    break
    nexats = int(excl.sum())
    Ndegf = 3 * natom - nconstr
    Ndegfree = Ndegf - 3 * nexats + exclshk
    Ndegf_solvent = Ndegf - 3 * nsol + solute_constraints
    Ndegf_solute = Ndegf - Ndegf_solvent
    Ndegfree_solvent = 3 * (natom - nsol) - (nconstr - solute_constraints)
    Ndegfree_solute = Ndegfree - Ndegfree_solvent
    separate_scaling = inp["separate_scaling"]
    detail = True
    if Ndegfree_solvent * Ndegfree_solute == 0:
        detail = False
        separate_scaling = False
    shake_first = np.cumsum([0] + [len(m) for m in shake_mols]).astype(np.int32)
    flat = [c for m in shake_mols for c in m]
    shake_i = np.array([c[0] for c in flat], dtype=np.int32)
    shake_j = np.array([c[1] for c in flat], dtype=np.int32)
    shake_d2 = np.array([c[2] for c in flat], dtype=np.float64)

    # --- make_qconn (src/md.f90:9582-9611) and nbqqlist (9691-9804); their
    # inputs are kept on the System so that the oracle's restatement can
    # rebuild the lists independently (tests/test_oracle_qconn.py)
    qconn_in = {
        "bnd": np.asarray(bnd[:top["nbonds_solute"], :3], dtype=np.int32).reshape(-1, 3),
        "qbnd": np.asarray(qbnd, dtype=np.int32).reshape(-1, 2 + S),
        "exspec": np.array([[i, j] + [int(bool(x)) for x in f[:S]] for i, j, f in exspec], dtype=np.int32).reshape(-1, 2 + S),
        "soft": np.array(soft_pairs, dtype=np.int32).reshape(-1, 2),
        "els_ij": np.array([(a, b) for a, b, _ in el_scale], dtype=np.int32).reshape(-1, 2),
        "els_v": np.array([list(v[:S]) for _, _, v in el_scale], dtype=np.float64).reshape(-1, S),
        "qvdw": np.int32(1 if qvdw_flag else 0),
    }
    qconn = np.full((S, nsol, nq), 9, dtype=np.int8)
    adj_cl: dict[int, list[int]] = {}
    for b in range(top["nbonds_solute"]):
        i, j, cod = bnd[b]
        if cod == 0:
            continue
        adj_cl.setdefault(i, []).append(j)
        adj_cl.setdefault(j, []).append(i)
    for iq in range(nq):
        qconn[:, iqseq[iq], iq] = 1
    for s in range(S):
        adj = {k: list(v) for k, v in adj_cl.items()}
        for q in qbnd:
            if q[2 + s] > 0:
                adj.setdefault(q[0], []).append(q[1])
                adj.setdefault(q[1], []).append(q[0])
        for iq in range(nq):
            o = iqseq[iq]
            dq = deque([(o, 1)])
            while dq:
                cur, lev = dq.popleft()
                if lev >= 4:
                    continue
                for nb in adj.get(cur, []):
                    if qconn[s, nb, iq] > lev + 1:
                        qconn[s, nb, iq] = lev + 1
                        dq.append((nb, lev + 1))
    for i, j, f in exspec:
        for (a, b) in ((i, j), (j, i)):
            iq = iqatom[a]
            if iq >= 0:
                for s in range(S):
                    if f[s]:
                        qconn[s, b, iq] = 0
    nbqq = {"iq": [], "j": [], "jq": [], "lj": [], "els": []}
    per_state: list[list[tuple]] = [[] for _ in range(S)]
    for iq in range(nq - 1):
        for jq in range(iq + 1, nq):
            j = iqseq[jq]
            for s in range(S):
                c = qconn[s, j, iq]
                if c > 3:
                    if c == 4:
                        lj = 3
                    elif not qvdw_flag:
                        lj = int(ljcod[iac[iqseq[iq]], iac[j]])
                    else:
                        lj = 2 if ((iq, jq) in soft_pairs or (jq, iq) in soft_pairs) else 1
                    els = 1.0
                    for a, b, v in el_scale:
                        if (a, b) in ((iq, jq), (jq, iq)):
                            els = v[s]
                            break
                    per_state[s].append((iq, j, jq, lj, els))
    for j in range(nsol):
        if iqatom[j] >= 0:
            continue
        if np.any(qconn[:, j, :] <= 3):
            for iq in range(nq):
                for s in range(S):
                    c = qconn[s, j, iq]
                    if c >= 4:
                        lj = 3 if c == 4 else (1 if qvdw_flag else int(ljcod[iac[iqseq[iq]], iac[j]]))
                        per_state[s].append((iq, j, -1, lj, 1.0))
    nbqq_count = [len(p) for p in per_state]
    for p in per_state:
        for row in p:
            for k, key in enumerate(("iq", "j", "jq", "lj", "els")):
                nbqq[key].append(row[k])
    nbqq = {k: np.array(v) for k, v in nbqq.items()}
    qp_skip = np.zeros(natom, dtype=np.uint8)
    if nq:
        qp_skip[:nsol] = np.any(qconn <= 3, axis=(0, 2))
    qp14 = [(iq, j) for j in range(nsol) if not qp_skip[j] for iq in range(nq) if qconn[0, j, iq] == 4]

    # --- shrink_topology (src/md.f90: order-preserving swaps of the reference)
    bnd, nb_sol = _shrink(bnd, top["nbonds_solute"], lambda r: r[2] <= 0)
    ang, na_sol = _shrink(ang, top["nangles_solute"], lambda r: r[3] == 0)
    tor, nt_sol = _shrink(tor, top["ntors_solute"], lambda r: r[4] == 0)
    imp, ni_sol = _shrink(imp, top["nimps_solute"], lambda r: r[4] == 0)
    anglib = top["anglib"].copy()
    anglib[:, 1] *= DEG2RAD
    t32 = top["torlib"].astype(np.float32)
    torlib = np.stack([t32[:, 0], t32[:, 1], (DEG2RAD * t32[:, 2].astype(np.float64)).astype(np.float32),
                       (1.0 / t32[:, 3].astype(np.float64)).astype(np.float32)], axis=1)
    i32 = top["implib"].astype(np.float32)
    implib = np.stack([i32[:, 0], (DEG2RAD * i32[:, 1].astype(np.float64)).astype(np.float32)], axis=1)

    sc_lookup = np.zeros((nq, natyps + nq, S), dtype=np.float64)
    ns = nsol
    chg_solv = crg[ns:ns + 3].copy()
    aLJ_solv = np.array([avdw[iac[ns + k], 0:2] for k in range(3)])
    bLJ_solv = np.array([bvdw[iac[ns + k], 0:2] for k in range(3)])
    x = xtop.copy()

    # --- thermostat / integrator ([MD], initialize src/md.f90:4648-4705)
    thermo = {"berendsen": 0, "langevin": 1, "nose-hoover": 2}.get(str(inp["thermostat"]).lower())
    if thermo is None:
        raise ValueError(f"unknown thermostat {inp['thermostat']}")
    integ = {"leap-frog": 0, "velocity-verlet": 1}.get(str(inp["integrator"]).lower())
    if integ is None:
        raise ValueError(f"unknown integrator {inp['integrator']}")
    tau_T = TIME_UNIT * inp["bath_coupling"]
    friction = inp.get("langevin_friction") if inp.get("langevin_friction") is not None else 1.0 / tau_T
    kbT = BOLTZ * inp["temperature"]
    nhq = inp.get("nose_hoover_mass") if inp.get("nose_hoover_mass") is not None else kbT / (tau_T * tau_T)

    # --- sequence restraints (0-based atoms)
    rs = inp.get("sequence_restraints", [])
    rstseq_ij = np.array([(a - 1, b - 1) for a, b, _, _, _ in rs], dtype=np.int32).reshape(-1, 2)
    rstseq_fk = np.array([fk for _, _, fk, _, _ in rs], dtype=np.float64)
    rstseq_flags = np.array([(ih, tc) for _, _, _, ih, tc in rs], dtype=np.int32).reshape(-1, 2)

    # --- water polarisation shells (wat_sphere / wat_shells, src/md.f90:18106-18368)
    wpol = bool(inp["polarisation"]) and natom > nsol and not use_pbc
    fkwpol = inp.get("polarisation_force", -1.0) if inp.get("polarisation_force", -1.0) != -1.0 else 20.0
    wshell = np.zeros((0, 4))
    if wpol:
        crgQtot = 0.0
        if inp.get("charge_correction", inp["polarisation"]):
            for iq in range(nq):
                for s_ in range(S):
                    crgQtot += qcrg[iq, s_] / sq * lam[s_]
        # the water dipole from the last bond and angle of the topology
        bcod = int(top["bnd"][-1][2]) - 1
        acod = int(top["ang"][-1][3]) - 1
        mu_w = -(crg[nsol] / sq) * top["bondlib"][bcod][1] * math.cos(top["anglib"][acod][1] * DEG2RAD / 2.0)
        drs = 3.0001 / 0.5
        nsh = int(-0.5 + math.sqrt(2.0 * drs + 0.25))
        rows = []
        rout = rwat
        pi = 4.0 * math.atan(1.0)
        for k in range(1, nsh + 1):
            dr = 0.5 * k
            ri = rout - dr
            rshell = (0.5 * (rout ** 3 + ri ** 3)) ** (1.0 / 3.0)
            cstb = crgQtot * 0.98750 / (0.0335 * mu_w * 4.0 * pi * rshell ** 2)
            rows.append((rout, dr, cstb, 0.0))
            rout = rout - dr
        wshell = np.array(rows, dtype=np.float64).reshape(-1, 4)
    # --- the other p_restrain restraints (0-based atoms; state 0 = every state)
    def _state(st, what):
        if st < 0 or st > S:
            raise ValueError(f"{what}: state {st} outside 0..{S}")
        return st
    pos = inp.get("atom_restraints", [])
    dis = inp.get("distance_restraints", [])
    ang_r = inp.get("angle_restraints", [])
    wal = [] if use_pbc else inp.get("wall_restraints", [])
    rst_extra = dict(
        rstpos_i=np.array([(r[0] - 1, _state(r[7], "atom restraint")) for r in pos], np.int32).reshape(-1, 2),
        rstpos_x=np.array([r[1:7] for r in pos], np.float64).reshape(-1, 6),
        rstdis_i=np.array([(r[0] - 1, r[1] - 1, _state(r[5], "distance restraint")) for r in dis], np.int32).reshape(-1, 3),
        rstdis_p=np.array([r[2:5] for r in dis], np.float64).reshape(-1, 3),
        rstang_i=np.array([(r[0] - 1, r[1] - 1, r[2] - 1, _state(r[5], "angle restraint")) for r in ang_r],
                          np.int32).reshape(-1, 4),
        rstang_p=np.array([r[3:5] for r in ang_r], np.float64).reshape(-1, 2),
        rstwal_i=np.array([(r[0] - 1, r[1] - 1, r[6]) for r in wal], np.int32).reshape(-1, 3),
        rstwal_p=np.array([r[2:6] for r in wal], np.float64).reshape(-1, 4))

    # --- periodic box: Q-atom switching atom and the molecules put_back_in_box moves
    qswitch = -1
    if use_pbc and nq:
        if fep is None or fep.get("qswitch") is None:
            raise ValueError("a periodic box with Q atoms needs [PBC] switching_atom in the FEP file")
        qswitch = int(fep["qswitch"]) - 1
    if use_pbc and inp["Rcq"] < 0:
        raise ValueError("q_atom < 0 (all atoms on the Q lists) is not supported in a periodic box")
    nsolvent_mol = int(top.get("nres", 0)) - int(top.get("nres_solute", top.get("nres", 0)))
    box = dict(use_pbc=int(use_pbc), boxlength=np.asarray(top.get("boxlength", np.zeros(3)), dtype=np.float64),
               boxcentre=np.asarray(top.get("boxcentre", np.zeros(3)), dtype=np.float64), qswitch=qswitch,
               put_solute_back=int(inp.get("put_solute_back_in_box", False)),
               put_solvent_back=int(inp.get("put_solvent_back_in_box", False)),
               rigid_box_centre=int(inp.get("rigid_box_centre", False)),
               istart_mol=np.asarray(istart[:-1], dtype=np.int32), nsolute_mol=nmol - nsolvent_mol)
    return System(
        **box, **rst_extra,
        natom=natom, nat_solute=nsol, natyps=natyps, ncgp_solute=ncgp_solute, nqat=nq, nstates=S,
        x=x, v=np.zeros(3 * natom), xtop=xtop, crg=crg, iac=iac, excl=excl, shell=shell, iqatom=iqatom,
        mass=mass, avdw=avdw, bvdw=bvdw, ljcod=ljcod, el14_scale=top["el14_scale"], ff_type=top["ff_type"],
        ivdw_rule=int(top["ivdw_rule"]),
        chg_solv=chg_solv, aLJ_solv=aLJ_solv, bLJ_solv=bLJ_solv,
        cgp_first=cgp_first, cgp_last=cgp_last, cgp_switch=cgp_switch, cgpatom=cgpatom,
        excl_pairs=np.array(sorted(excl_set), dtype=np.int32).reshape(-1, 2),
        pairs14=np.array(sorted(p14_set), dtype=np.int32).reshape(-1, 2),
        iqseq=iqseq.astype(np.int32), qcrg=qcrg, qvdw_flag=qvdw_flag, qiac=qiac, qavdw=qavdw, qbvdw=qbvdw,
        sc_lookup=sc_lookup, lambdas=lam[:S] + [0.0] * (MAX_STATES - S),
        qp_skip=qp_skip, qp14_pairs=np.array(qp14, dtype=np.int32).reshape(-1, 2),
        nbqq_count=nbqq_count + [0] * (MAX_STATES - S), nbqq=nbqq, qconn_in=qconn_in,
        qbnd=qbnd, qbondlib=qbondlib, qang=qang, qanglib=qanglib, qtor=qtor, qtorlib=qtorlib,
        qimp=qimp, qimplib=qimplib,
        bnd=bnd, nbonds_solute=nb_sol, bondlib=top["bondlib"], ang=ang, nangles_solute=na_sol, anglib=anglib,
        tor=tor, ntors_solute=nt_sol, torlib=torlib, imp=imp, nimps_solute=ni_sol, implib=implib,
        shake_first=shake_first, shake_i=shake_i, shake_j=shake_j, shake_dist2=shake_d2,
        offd=offd, xpcent=top["xpcent"], xwcent=top["xwcent"], rexcl_o=rexcl_o, rwat=rwat,
        fk_wsphere=fk_wsphere, Dwmz=Dwmz, awmz=awmz, fk_pshell=inp["shell_force"], fk_fix=fk_fix,
        wpol_restr=wpol, fkwpol=fkwpol, wshell=wshell, itdis_update=100,
        rstseq_ij=rstseq_ij, rstseq_fk=rstseq_fk, rstseq_flags=rstseq_flags, heavy=heavy.astype(np.uint8),
        excluded_freeze=int(inp.get("excluded_freeze", False)),
        thermostat=thermo, integrator=integ, friction=friction, langevin_gauss=int(inp.get("langevin_random", False)),
        rand_state=int(inp["random_seed"]), nhchains=int(inp.get("nhchains", 10)), nhq=nhq,
        Rcpp=inp["Rcpp"], Rcww=inp["Rcww"], Rcpw=inp["Rcpw"], Rcq=inp["Rcq"], RcLRF=inp["RcLRF"],
        use_LRF=inp["lrf"], dt=TIME_UNIT * inp["stepsize"], Temp0=inp["temperature"],
        tau_T=tau_T, separate_scaling=separate_scaling, NBcycle=inp["non_bond"],
        Ndegf=Ndegf, Ndegfree=Ndegfree, Ndegf_solvent=Ndegf_solvent, Ndegfree_solvent=Ndegfree_solvent,
        Ndegf_solute=Ndegf_solute, Ndegfree_solute=Ndegfree_solute, detail_temps=detail,
        any_atom_lists=0 if int(top.get("iuse_switch_atom", 1)) == 1 else 1,
        Tmaxw=inp["initial_temperature"], seed=inp["random_seed"], nsteps=inp["steps"],
    )


def _shrink(rows: np.ndarray, nsol: int, drop) -> tuple[np.ndarray, int]:
    """shrink_topology's in-place removal: a dropped solute row is replaced by
    the last solute row, which is replaced by the last row overall."""
    rows = [r.copy() for r in rows]
    n = len(rows)
    i = 0
    while i < n:
        if drop(rows[i]):
            if i < nsol:
                rows[i] = rows[nsol - 1]
                rows[nsol - 1] = rows[n - 1]
                nsol -= 1
            else:
                rows[i] = rows[n - 1]
            n -= 1
            continue
        i += 1
    width = rows[0].shape[0] if rows else 0
    out = np.array(rows[:n], dtype=np.int32).reshape(n, width) if n else np.zeros((0, max(width, 1)), dtype=np.int32)
    return out, nsol
