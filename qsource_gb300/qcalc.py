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


def rdf_normalise(counts: np.ndarray, radius: float, nframes: int, n1: int) -> np.ndarray:
    """RDF_finalize (calc_rdf.f90): counts / shell volume / frames / mask-1 atoms."""
    nb = len(counts)
    pi = 4.0 * np.arctan(1.0)
    j = np.arange(1, nb + 1, dtype=np.float64)
    vol = 4.0 * pi / 3.0 * ((j * radius / nb) ** 3 - ((j - 1) * radius / nb) ** 3)
    return counts / vol / nframes / n1
