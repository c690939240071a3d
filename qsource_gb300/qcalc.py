"""qcalc-style trajectory analysis: DCD frames in the reference's layout and
the device calculations of include/qgpu.h (qgpu_calc_*).

DCD layout (src/trj.f90, Fortran unformatted sequential records, each framed by
a 4-byte length before and after the payload):
  record 1 (trj_create :188, type REC1 :12-19): char[4] 'CORD', then 20 int32:
      n_frames, n_steps_before, interval, n_steps, interval_velcheck (0), 2
      unused, n_degf, n_fixed (0), unused, const_p (0), 8 unused,
      charmm_version (0)
  record 2 (:189): int32 2 + mask_rows, char[80] 'Q DCD trajectory version
      5.6', char[80] topology, mask_rows x char[80] atom-mask rows ('all' when
      qdyn's input has no [trajectory_atoms], md.f90:5001-5004)
  record 3 (:190): int32 atoms in the mask
  per frame (trj_write :211-229): three records of float32, x, y, z of the
      masked atoms.
"""
from __future__ import annotations

import ctypes as C
import struct

import numpy as np

from . import abi

TITLE = "Q DCD trajectory version 5.6"


def _rec(f, payload: bytes) -> None:
    n = struct.pack("<i", len(payload))
    f.write(n + payload + n)


def _read_rec(f) -> bytes:
    h = f.read(4)
    if len(h) < 4:
        raise EOFError
    (n,) = struct.unpack("<i", h)
    b = f.read(n)
    (m,) = struct.unpack("<i", f.read(4))
    if m != n or len(b) != n:
        raise ValueError("corrupt Fortran record")
    return b


def write_dcd(path: str, frames: np.ndarray, *, steps_before: int = 0, interval: int = 1, n_steps: int | None = None,
              n_degf: int = 0, topology: str = "", mask_rows=("all",), atoms: np.ndarray | None = None) -> None:
    """frames: [nframes, natom*3] (or [nframes, natom, 3]) FP64 coordinates;
    atoms: the 0-based atoms of the mask (all atoms when None)."""
    fr = np.asarray(frames, dtype=np.float64)
    nf = fr.shape[0]
    fr = fr.reshape(nf, -1, 3)
    if atoms is not None:
        fr = fr[:, np.asarray(atoms, dtype=np.int64), :]
    na = fr.shape[1]
    if n_steps is None:
        n_steps = nf * interval
    ints = [nf, steps_before, interval, n_steps, 0, 0, 0, n_degf, 0, 0, 0] + [0] * 8 + [0]
    rows = [TITLE, topology] + list(mask_rows)
    with open(path, "wb") as f:
        _rec(f, b"CORD" + struct.pack("<20i", *ints))
        _rec(f, struct.pack("<i", len(rows)) + b"".join(r.encode()[:80].ljust(80) for r in rows))
        _rec(f, struct.pack("<i", na))
        for k in range(nf):
            for c in range(3):
                _rec(f, fr[k, :, c].astype("<f4").tobytes())


def read_dcd(path: str):
    """Returns (header dict, frames [nframes, natom*3] FP64 of the float32
    values, as trj_read_masked copies them)."""
    out = []
    with open(path, "rb") as f:
        r1 = _read_rec(f)
        if r1[:4] != b"CORD":
            raise ValueError("not a DCD coordinate trajectory")
        ints = struct.unpack("<20i", r1[4:84])
        r2 = _read_rec(f)
        (nrows,) = struct.unpack("<i", r2[:4])
        rows = [r2[4 + 80 * k:4 + 80 * (k + 1)].decode().rstrip() for k in range(nrows)]
        if not rows or not rows[0].startswith("Q DCD trajectory"):
            raise ValueError("not a Q DCD trajectory")
        (na,) = struct.unpack("<i", _read_rec(f))
        while True:
            try:
                xyz = [np.frombuffer(_read_rec(f), dtype="<f4") for _ in range(3)]
            except EOFError:
                break
            out.append(np.stack(xyz, axis=1).astype(np.float64).reshape(-1))
    head = {"n_frames": ints[0], "n_steps_before": ints[1], "interval": ints[2], "n_steps": ints[3],
            "n_degf": ints[7], "title": rows[0], "topology": rows[1] if len(rows) > 1 else "",
            "mask_rows": rows[2:], "atoms": na}
    return head, np.array(out).reshape(len(out), 3 * na)


class Calc:
    """The device calculations over a set of frames (qgpu_calc_*)."""

    def __init__(self, lib=None):
        self.lib = lib or abi.load_library()

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(abi.last_error(self.lib))

    @staticmethod
    def _frames(frames):
        fr = np.ascontiguousarray(frames, dtype=np.float64)
        nf = fr.shape[0]
        return fr.reshape(nf, -1), nf, fr.reshape(nf, -1).shape[1] // 3

    def rms(self, frames, mask, xref) -> np.ndarray:
        fr, nf, na = self._frames(frames)
        m = np.ascontiguousarray(mask, dtype=np.int32)
        x0 = np.ascontiguousarray(xref, dtype=np.float64)
        out = np.zeros(nf)
        self._check(self.lib.qgpu_calc_rms(abi.ptr(fr), nf, na, abi.ptr(m), len(m), abi.ptr(x0), abi.ptr(out)))
        return out

    def rmsf(self, frames, mask) -> np.ndarray:
        """RMS fluctuation of the mask after each frame (calc_rmsf.f90)."""
        fr, nf, na = self._frames(frames)
        m = np.ascontiguousarray(mask, dtype=np.int32)
        out = np.zeros(nf)
        self._check(self.lib.qgpu_calc_rmsf(abi.ptr(fr), nf, na, abi.ptr(m), len(m), abi.ptr(out)))
        return out

    def fit(self, frames, nsol: int, mask, mass, xref):
        """Frames with their solute superposed on xref (calc_fit.f90), and the
        per-frame status (0 fitted; 1, 2 only moved, as qcalc)."""
        fr, nf, na = self._frames(frames)
        m = np.ascontiguousarray(mask, dtype=np.int32)
        ms = np.ascontiguousarray(mass, dtype=np.float64)
        x0 = np.ascontiguousarray(xref, dtype=np.float64)
        out = np.zeros((nf, 3 * na))
        st = np.zeros(nf, dtype=np.int32)
        self._check(self.lib.qgpu_calc_fit(abi.ptr(fr), nf, na, int(nsol), abi.ptr(m), len(m), abi.ptr(ms),
                                           abi.ptr(x0), abi.ptr(out), abi.ptr(st)))
        return out, st

    def com(self, frames, mask, mass) -> np.ndarray:
        fr, nf, na = self._frames(frames)
        m = np.ascontiguousarray(mask, dtype=np.int32)
        ms = np.ascontiguousarray(mass, dtype=np.float64)
        out = np.zeros((nf, 3))
        self._check(self.lib.qgpu_calc_com(abi.ptr(fr), nf, na, abi.ptr(m), len(m), abi.ptr(ms), abi.ptr(out)))
        return out

    def com_ke(self, frames, mask, mass, frame_length: float) -> np.ndarray:
        """Per frame (translational, rotational) kinetic energy of the mask's
        centre of mass, kcal/mol (calc_com_ke.f90); frame_length in fs."""
        fr, nf, na = self._frames(frames)
        m = np.ascontiguousarray(mask, dtype=np.int32)
        ms = np.ascontiguousarray(mass, dtype=np.float64)
        out = np.zeros((nf, 2))
        self._check(self.lib.qgpu_calc_com_ke(abi.ptr(fr), nf, na, abi.ptr(m), len(m), abi.ptr(ms),
                                              C.c_double(frame_length), abi.ptr(out)))
        return out

    def geom(self, frames, measurements) -> np.ndarray:
        """measurements: list of atom tuples (2 distance, 3 angle, 4 torsion)."""
        fr, nf, na = self._frames(frames)
        at = np.zeros((len(measurements), 4), dtype=np.int32)
        kind = np.array([len(m) for m in measurements], dtype=np.int32)
        for k, m in enumerate(measurements):
            at[k, :len(m)] = m
        out = np.zeros((nf, len(measurements)))
        self._check(self.lib.qgpu_calc_geom(abi.ptr(fr), nf, na, len(measurements), abi.ptr(at), abi.ptr(kind),
                                            abi.ptr(out)))
        return out

    def rdf_counts(self, frames, mask1, mask2, radius: float, nbins: int, box=None) -> np.ndarray:
        fr, nf, na = self._frames(frames)
        m1 = np.ascontiguousarray(mask1, dtype=np.int32)
        m2 = np.ascontiguousarray(mask2, dtype=np.int32)
        b = None if box is None else np.ascontiguousarray(box, dtype=np.float64)
        out = np.zeros(nbins, dtype=np.int64)
        self._check(self.lib.qgpu_calc_rdf(abi.ptr(fr), nf, na, abi.ptr(m1), len(m1), abi.ptr(m2), len(m2),
                                           C.c_double(radius), nbins, abi.ptr(b) if b is not None else None,
                                           abi.ptr(out)))
        return out

    def nb(self, frames, lst: "NbList", lambdas=None) -> np.ndarray:
        """Per frame and list (Vlj, Vel) (calc_nb.f90 nb_calc_lists), shape
        [nframes, nlist, 2]; lambdas: one weight per state (None: all 1)."""
        fr, nf, na = self._frames(frames)
        S = lst.AA.shape[1]
        lam = np.ones(S) if lambdas is None else np.ascontiguousarray(lambdas, dtype=np.float64)
        if lam.shape != (S,):
            raise ValueError(f"{S} states in the list, {lam.size} lambdas")
        n = len(lst.pairs)
        st = np.ascontiguousarray(lst.starts, dtype=np.int64)
        pr = np.ascontiguousarray(lst.pairs, dtype=np.int32).reshape(-1) if n else np.zeros(2, np.int32)
        dd = lambda a: np.ascontiguousarray(a, dtype=np.float64).reshape(-1) if n else np.zeros(S)
        A, B, Q = dd(lst.AA), dd(lst.BB), dd(lst.qq)
        nl = len(st) - 1
        out = np.zeros((nf, nl, 2))
        self._check(self.lib.qgpu_calc_nb(abi.ptr(fr), nf, na, nl, abi.ptr(st), abi.ptr(pr), S, abi.ptr(lam),
                                          abi.ptr(A), abi.ptr(B), abi.ptr(Q), int(lst.arith), abi.ptr(out)))
        return out


class NbList:
    """Pair lists of nonbonded calculations and their per-state LJ and charge
    products (AA, BB, qq: [npair, nstates]); list l is pairs
    [starts[l], starts[l+1])."""

    def __init__(self, pairs, AA, BB, qq, arith, starts=None):
        self.pairs, self.AA, self.BB, self.qq, self.arith = pairs, AA, BB, qq, bool(arith)
        self.starts = np.array([0, len(pairs)], dtype=np.int64) if starts is None else np.asarray(starts, np.int64)


def nb_qp_make_lists(g, residues, qmask, fep: bool = False) -> NbList:
    """nb_qp_add (calc_nb.f90:778-938): one list per residue, the residue's
    atoms against the Q-atom mask (nb_make_list each); residues: the atom
    index arrays of the residues, in order."""
    parts = [nb_make_list(g, r, qmask, fep=fep) for r in residues]
    S = int(g.nstates) if fep else 1
    starts = np.concatenate([[0], np.cumsum([len(p.pairs) for p in parts])]).astype(np.int64)
    cat = lambda k, shape: np.concatenate([getattr(p, k) for p in parts]) if parts else np.zeros(shape)
    return NbList(cat("pairs", (0, 2)).astype(np.int32), cat("AA", (0, S)), cat("BB", (0, S)), cat("qq", (0, S)),
                  int(getattr(g, "ivdw_rule", 1)) == 2, starts)


def nb_make_list(g, mask1, mask2, fep: bool = False, chunk: int = 1 << 22) -> NbList:
    """nb_make_list (calc_nb.f90:334-759) for the system g: every pair of a
    mask-1 atom and a mask-2 atom (both ascending, mask-1 atom outer), except
      * pairs whose first atom is not below the second when the second is in
        both masks (:401-410);
      * pairs of atoms that share an angle of the topology (:412-425).
    LJ code: the type pair code (1, or 2 for the polar pairs), 3 for a 1-4
    pair (:442-461).  Per state, AA = a1*a2 (geometric rule) or a1 + a2
    (arithmetic), BB = b1*b2 at that code; with fep a Q atom (a solute atom
    with a Q index) takes its state's Q type and charge, and for code 2 with a
    non-Q partner its code-1 parameters (:463-683).  Charge products: with fep
    q1*q2, times the 1-4 scale for 1-4 pairs (:684-740); without fep
    crg1*crg2*el14_scale for every pair (:742).  The system's charges carry
    sqrt(Coulomb constant).  The pairs are built chunk by chunk of mask-1
    atoms (about `chunk` pairs at a time)."""
    natom, nsol = int(g.natom), int(g.nat_solute)
    in1 = np.zeros(natom, bool); in1[np.asarray(mask1, dtype=np.int64)] = True
    in2 = np.zeros(natom, bool); in2[np.asarray(mask2, dtype=np.int64)] = True
    g1, g2 = np.flatnonzero(in1), np.flatnonzero(in2)
    mutual = in1 & in2
    N = np.int64(natom)

    def keys(a, b):
        a, b = np.asarray(a, np.int64), np.asarray(b, np.int64)
        return np.minimum(a, b) * N + np.maximum(a, b)

    ang = np.asarray(g.ang).reshape(len(g.ang), -1)[:, :3].astype(np.int64) if len(g.ang) else np.zeros((0, 3), np.int64)
    akeys = np.unique(np.concatenate([keys(ang[:, 0], ang[:, 1]), keys(ang[:, 0], ang[:, 2]),
                                      keys(ang[:, 1], ang[:, 2])]))
    p14 = np.asarray(g.pairs14, dtype=np.int64).reshape(-1, 2)
    pkeys = np.unique(keys(p14[:, 0], p14[:, 1]))
    iac = np.asarray(g.iac, dtype=np.int64)
    avdw, bvdw = np.asarray(g.avdw, np.float64), np.asarray(g.bvdw, np.float64)
    ljcod = np.asarray(g.ljcod, dtype=np.int64)
    crg = np.asarray(g.crg, np.float64)
    arith = int(getattr(g, "ivdw_rule", 1)) == 2
    el14 = float(g.el14_scale)
    S = int(g.nstates) if fep else 1
    iqatom = np.asarray(g.iqatom, dtype=np.int64)
    isq = np.zeros(natom, bool)
    if fep:
        isq[:nsol] = iqatom[:nsol] >= 0
    qiac = np.asarray(g.qiac, dtype=np.int64).reshape(-1, int(g.nstates)) if fep else None
    qcrg = np.asarray(g.qcrg, np.float64).reshape(-1, int(g.nstates)) if fep else None
    qavdw, qbvdw = np.asarray(g.qavdw, np.float64), np.asarray(g.qbvdw, np.float64)

    def params(me, other, code, s):
        a = avdw[iac[me], code - 1]
        b = bvdw[iac[me], code - 1]
        q = crg[me].copy()
        if fep:
            qm = isq[me]
            if qm.any():
                m = me[qm]
                c = np.where((code[qm] == 2) & ~isq[other[qm]], 1, code[qm])
                t = qiac[iqatom[m], s]
                a[qm], b[qm], q[qm] = qavdw[t, c - 1], qbvdw[t, c - 1], qcrg[iqatom[m], s]
        return a, b, q

    out = {k: [] for k in ("p", "A", "B", "Q")}
    rows = max(1, chunk // max(1, len(g2)))
    for r0 in range(0, len(g1), rows):
        J = np.repeat(g1[r0:r0 + rows], len(g2))
        K = np.tile(g2, len(g1[r0:r0 + rows]))
        key = keys(J, K)
        keep = ~((J >= K) & mutual[K]) & ~np.isin(key, akeys)
        J, K, key = J[keep], K[keep], key[keep]
        code = np.where(np.isin(key, pkeys), 3, ljcod[iac[J], iac[K]])
        A = np.empty((len(J), S)); B = np.empty((len(J), S)); Q = np.empty((len(J), S))
        for s in range(S):
            a1, b1, q1 = params(J, K, code, s)
            a2, b2, q2 = params(K, J, code, s)
            A[:, s] = a1 + a2 if arith else a1 * a2
            B[:, s] = b1 * b2
            Q[:, s] = np.where(code == 3, q1 * q2 * el14, q1 * q2) if fep else q1 * q2 * el14
        out["p"].append(np.stack([J, K], 1)); out["A"].append(A); out["B"].append(B); out["Q"].append(Q)
    cat = lambda k, shape: np.concatenate(out[k]) if out[k] else np.zeros(shape)
    return NbList(cat("p", (0, 2)).astype(np.int32), cat("A", (0, S)), cat("B", (0, S)), cat("Q", (0, S)), arith)


def nb_averages(values) -> float:
    """The running average qcalc prints after the last frame (calc_nb.f90
    nb_calc :248-251): ave <- (ave*n + V)/(n + 1)."""
    ave, n = 0.0, 0
    for v in values:
        ave = (ave * n + float(v)) / (n + 1)
        n += 1
    return ave


def rdf_normalise(counts: np.ndarray, radius: float, nframes: int, n1: int) -> np.ndarray:
    """RDF_finalize (calc_rdf.f90): counts / shell volume / frames / mask-1 atoms."""
    nb = len(counts)
    pi = 4.0 * np.arctan(1.0)
    j = np.arange(1, nb + 1, dtype=np.float64)
    vol = 4.0 * pi / 3.0 * ((j * radius / nb) ** 3 - ((j - 1) * radius / nb) ** 3)
    return counts / vol / nframes / n1
