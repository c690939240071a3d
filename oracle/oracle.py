"""ctypes wrapper of the FP64 C oracle (oracle/qoracle.c) -- test infrastructure.

Builds liboracle on first use (make in this directory).  The engine never
imports this module; tests, smoke() and bench.py's CPU baseline do.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from qsource_gb300.abi import Energies, QEnergy, SystemDesc

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(_HERE, "_build", "libqoracle.so")
_lib = None


def build() -> str:
    """Compile qoracle.c with the flags of oracle/Makefile (gcc, no make needed)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cc = os.environ.get("CC", "gcc")
    subprocess.run([cc, "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-std=c11",
                    "-I" + os.path.join(os.path.dirname(_HERE), "include"), "-shared", "-o", LIB,
                    os.path.join(_HERE, "qoracle.c"), "-lm"], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        src = os.path.join(_HERE, "qoracle.c")
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
            build()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [C.POINTER(SystemDesc)]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_set_coords.argtypes = [vp, vp, vp]
        L.oracle_get_coords.argtypes = [vp, vp, vp]
        L.oracle_make_pair_lists.argtypes = [vp]
        L.oracle_get_list.restype = C.c_int64
        L.oracle_get_list.argtypes = [vp, C.c_int, vp, C.c_int64]
        L.oracle_get_list_shift.restype = C.c_int64
        L.oracle_get_list_shift.argtypes = [vp, C.c_int, vp, C.c_int64]
        L.oracle_get_lrf.argtypes = [vp, vp]
        L.oracle_pot_energy.argtypes = [vp, C.c_int, vp, C.POINTER(Energies), C.POINTER(QEnergy)]
        L.oracle_shake_arrays.restype = C.c_int
        L.oracle_shake_arrays.argtypes = [vp, vp, vp]
        L.oracle_maxwell.argtypes = [vp, C.c_double, C.c_int32]
        L.oracle_initial_shaking.restype = C.c_int
        L.oracle_initial_shaking.argtypes = [vp]
        L.oracle_stop_cm_translation.argtypes = [vp]
        L.oracle_temperature.argtypes = [vp, vp]
        L.oracle_offdiag.argtypes = [vp, vp, vp]
        L.oracle_md_run.restype = C.c_int
        L.oracle_md_run.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(Energies), C.POINTER(QEnergy), vp]
        L.oracle_get_energies.argtypes = [vp, C.POINTER(Energies), C.POINTER(QEnergy)]
        L.oracle_final_energy.argtypes = [vp, C.c_int, C.POINTER(Energies), C.POINTER(QEnergy)]
        L.oracle_rand_state.restype = C.c_int32
        L.oracle_rand_state.argtypes = [vp]
        L.oracle_put_back_in_box.argtypes = [vp]
        L.oracle_qconn.restype = C.c_int
        L.oracle_qconn.argtypes = [C.c_int] * 3 + [vp] * 4 + [C.c_int, C.c_int, vp, C.c_int, vp, C.c_int, vp, C.c_int,
                                                       C.c_int, vp, C.c_int, vp, vp, vp, C.c_int] + [vp] * 9
        L.oracle_qfep_fep.restype = C.c_int
        L.oracle_qfep_fep.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.c_int, C.c_double, C.c_int, vp, vp, vp, vp]
        L.oracle_sizeof_desc.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


LIST_NAMES = {"pp": 0, "pw": 1, "ww": 2, "qp": 3, "qw": 4}


class Oracle:
    """One trajectory of the FP64 reference restatement."""

    def __init__(self, system):
        self.system = system
        self._desc = system.desc()
        self.L = lib()
        self.h = self.L.oracle_create(C.byref(self._desc))
        self.S = system.nstates
        self.N = system.natom

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.L.oracle_destroy(self.h)
        except Exception:
            pass

    def set_coords(self, x=None, v=None):
        self.L.oracle_set_coords(self.h, _p(None if x is None else np.ascontiguousarray(x, np.float64)),
                                 _p(None if v is None else np.ascontiguousarray(v, np.float64)))

    def coords(self):
        x = np.zeros(3 * self.N); v = np.zeros(3 * self.N)
        self.L.oracle_get_coords(self.h, _p(x), _p(v))
        return x, v

    def make_pair_lists(self):
        self.L.oracle_make_pair_lists(self.h)

    def get_list(self, name: str) -> np.ndarray:
        w = LIST_NAMES[name]
        n = self.L.oracle_get_list(self.h, w, None, 0)
        out = np.zeros((max(n, 1), 3), dtype=np.int32)
        self.L.oracle_get_list(self.h, w, _p(out), n)
        return out[:n]

    def get_list_shift(self, name: str) -> np.ndarray:
        """Records of a list as rows (i, j, si, sj): si, sj the atoms whose
        difference fixes the periodic shift (-1 in a sphere)."""
        w = LIST_NAMES[name]
        n = self.L.oracle_get_list_shift(self.h, w, None, 0)
        out = np.zeros((max(n, 1), 4), dtype=np.int32)
        self.L.oracle_get_list_shift(self.h, w, _p(out), n)
        return out[:n]

    def get_lrf(self) -> np.ndarray:
        out = np.zeros((len(self.system.cgp_first), 43))
        self.L.oracle_get_lrf(self.h, _p(out))
        return out

    def pot_energy(self, terms: int = 0x1F):
        d = np.zeros(3 * self.N)
        E = Energies()
        EQ = (QEnergy * max(self.S, 1))()
        self.L.oracle_pot_energy(self.h, terms, _p(d), C.byref(E), EQ)
        return d, E.as_dict(), [EQ[s].as_dict() for s in range(self.S)]

    def shake(self, xx, x) -> int:
        return self.L.oracle_shake_arrays(self.h, _p(xx), _p(x))

    def maxwell(self, T: float, seed: int):
        self.L.oracle_maxwell(self.h, T, seed)

    def initial_shaking(self) -> int:
        return self.L.oracle_initial_shaking(self.h)

    def stop_cm_translation(self):
        self.L.oracle_stop_cm_translation(self.h)

    def temperature(self):
        out = np.zeros(4)
        self.L.oracle_temperature(self.h, _p(out))
        return out

    def offdiag(self):
        n = len(self.system.offd)
        H = np.zeros(max(n, 1)); r = np.zeros(max(n, 1))
        self.L.oracle_offdiag(self.h, _p(H), _p(r))
        return H[:n], r[:n]

    def put_back_in_box(self):
        self.L.oracle_put_back_in_box(self.h)

    def rand_state(self) -> int:
        """The randm state the next random number continues from."""
        return int(self.L.oracle_rand_state(self.h))

    def final_energy(self, terms: int = 0x1F):
        """Lists and energies after an MD run (the reference's FINAL report)."""
        E = Energies()
        EQ = (QEnergy * max(self.S, 1))()
        self.L.oracle_final_energy(self.h, terms, C.byref(E), EQ)
        return E.as_dict(), [EQ[s].as_dict() for s in range(self.S)]

    def md_run(self, nsteps: int, terms: int = 0x1F):
        E = (Energies * nsteps)()
        EQ = (QEnergy * (nsteps * max(self.S, 1)))()
        T = np.zeros(nsteps)
        rc = self.L.oracle_md_run(self.h, nsteps, terms, E, EQ, _p(T))
        rows = [E[k].as_dict() for k in range(nsteps)]
        qrows = [[EQ[k * self.S + s].as_dict() for s in range(self.S)] for k in range(nsteps)]
        return rc, rows, qrows, T


def qfep_fep(paths, nstates: int, kT: float, nskip: int = 0):
    """qfep Part 1 on energy files in lambda order: (dgf, dgr, dG, npts)."""
    n = len(paths)
    arr = (C.c_char_p * n)(*[p.encode() for p in paths])
    dgf, dgr, dg = np.zeros(n), np.zeros(n), np.zeros(n)
    npts = np.zeros(n, dtype=np.int32)
    rc = lib().oracle_qfep_fep(n, arr, nstates, kT, nskip, _p(dgf), _p(dgr), _p(dg), _p(npts))
    if rc:
        raise RuntimeError("qfep: cannot read the energy files")
    return dgf, dgr, dg, npts


def qconn_lists(system):
    """make_qconn + nbqqlist restated in C (oracle_qconn) from the topology
    inputs kept on `system` (System.qconn_in): returns (qconn[ns, nsol, nq],
    per-state nbqq records [(iq, j, jq, lj, el_scale)], qp_skip[nsol],
    qp14 pairs [(iq, atom)])."""
    qi = system.qconn_in
    ns, nsol, nq = int(system.nstates), int(system.nat_solute), int(system.nqat)
    iqseq = np.ascontiguousarray(system.iqseq, np.int32)
    iqatom = np.ascontiguousarray(np.asarray(system.iqatom)[:nsol], np.int32)
    iac = np.ascontiguousarray(np.asarray(system.iac)[:nsol], np.int32)
    ljcod = np.ascontiguousarray(system.ljcod, np.int8)
    natyps = int(system.natyps)
    arr = {k: np.ascontiguousarray(qi[k], dt) for k, dt in
           (("bnd", np.int32), ("qbnd", np.int32), ("exspec", np.int32), ("soft", np.int32), ("els_ij", np.int32),
            ("els_v", np.float64))}
    cap = 8 * (nq * nq + nsol * nq) * ns + 16
    qconn = np.zeros((ns, nsol, max(nq, 1)), np.int8)
    count = np.zeros(ns, np.int32)
    o = {k: np.zeros(cap, np.int32) for k in ("iq", "j", "jq", "lj")}
    els = np.zeros(cap)
    qp_skip = np.zeros(max(nsol, 1), np.uint8)
    nqp14 = np.zeros(1, np.int32)
    qp14 = np.zeros(2 * cap, np.int32)
    rc = lib().oracle_qconn(nsol, nq, ns, _p(iqseq), _p(iqatom), _p(iac), _p(ljcod), natyps,
                            len(arr["bnd"]), _p(arr["bnd"]), len(arr["qbnd"]), _p(arr["qbnd"]),
                            len(arr["exspec"]), _p(arr["exspec"]), int(qi["qvdw"]), len(arr["soft"]), _p(arr["soft"]),
                            len(arr["els_ij"]), _p(arr["els_ij"]), _p(arr["els_v"]), _p(qconn), cap, _p(count),
                            _p(o["iq"]), _p(o["j"]), _p(o["jq"]), _p(o["lj"]), _p(els), _p(qp_skip), _p(nqp14), _p(qp14))
    if rc:
        raise RuntimeError("oracle_qconn: capacity")
    per_state, k = [], 0
    for s in range(ns):
        per_state.append([(int(o["iq"][k + r]), int(o["j"][k + r]), int(o["jq"][k + r]), int(o["lj"][k + r]),
                           float(els[k + r])) for r in range(count[s])])
        k += count[s]
    pairs = [(int(qp14[2 * r]), int(qp14[2 * r + 1])) for r in range(nqp14[0])]
    return qconn[:, :, :nq], per_state, qp_skip[:nsol], pairs


def md_frames(system, nsteps: int, ene_every: int, couplings):
    """One window's MD run with the oracle, as the frames of qdyn's energy
    file: at every recorded nonzero step (md_run writes frames there, src/
    md.f90:6630) the per-state totals EQ(s)%total, and for each coupling
    (i, j, A) of a constant off-diagonal element (mu = 0) the record
    (i, j, A, 0).  Returns (lambdas, frames) as qfep_ref.read_en does."""
    o = Oracle(system)
    o.temperature()
    rc, _, qrows, _ = o.md_run(nsteps)
    if rc:
        raise RuntimeError(f"oracle md_run status {rc}")
    S = int(system.nstates)
    lam = [float(system.lambdas[s]) for s in range(S)]
    frames = []
    for k in range(ene_every, nsteps, ene_every):
        frames.append(([qrows[k][s]["total"] for s in range(S)], [(i, j, a, 0.0) for i, j, a in couplings]))
    return lam, frames
