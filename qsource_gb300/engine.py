"""Python mirror of the engine's C-ABI (include/qgpu.h).

``Engine`` wraps one ``qgpu_handle`` holding a batch of trajectories.  Its
methods map one-to-one onto the drop-in call points of qdyn:

  make_pair_lists      -> qgpu_build_lists   (src/md.f90:5985)
  pot_energy(terms)    -> qgpu_forces        (src/md.f90:16015)
  shake(xx, x)         -> qgpu_shake         (src/md.f90:17581)
  run(nsteps)          -> qgpu_run           (the md_run loop, src/md.f90:6471-6664)

There is no CPU fallback: without the built CUDA library every call raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi


class QgpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"qgpu error {code} ({abi.STATUS.get(code, '?')}): {msg}")
        self.code = code


class Engine:
    def __init__(self, systems, lib_path: str | None = None):
        if not isinstance(systems, (list, tuple)):
            systems = [systems]
        self.systems = list(systems)
        self.lib = abi.load_library(lib_path)
        descs = (abi.SystemDesc * len(self.systems))()
        for k, s in enumerate(self.systems):
            descs[k] = s.desc()
        self._descs = descs
        h = C.c_void_p()
        self._check(self.lib.qgpu_create(descs, len(self.systems), C.byref(h)))
        self.h = h

    # ----------------------------------------------------------------- util
    def _check(self, rc: int):
        if rc != 0:
            raise QgpuError(rc, abi.last_error(self.lib))

    def close(self):
        if getattr(self, "h", None):
            self.lib.qgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def ntraj(self) -> int:
        return len(self.systems)

    def kernel_launches(self) -> int:
        return int(self.lib.qgpu_kernel_launches(self.h))

    # --------------------------------------------------------------- state
    def set_coords(self, traj: int, x=None, v=None):
        xa = None if x is None else np.ascontiguousarray(x, np.float64)
        va = None if v is None else np.ascontiguousarray(v, np.float64)
        self._check(self.lib.qgpu_set_coords(self.h, traj, abi.ptr(xa), abi.ptr(va)))

    def coords(self, traj: int = 0):
        n = 3 * self.systems[traj].natom
        x = np.zeros(n); v = np.zeros(n)
        self._check(self.lib.qgpu_get_coords(self.h, traj, abi.ptr(x), abi.ptr(v)))
        return x, v

    def set_coords_all(self, x=None, v=None):
        """Coordinates / velocities of every trajectory, back to back in
        trajectory order (qgpu_set_coords_all)."""
        xa = None if x is None else np.ascontiguousarray(x, np.float64)
        va = None if v is None else np.ascontiguousarray(v, np.float64)
        self._check(self.lib.qgpu_set_coords_all(self.h, abi.ptr(xa), abi.ptr(va)))

    def coords_all(self, x=None, v=None):
        """Every trajectory's x and v back to back (qgpu_get_coords_all); fills
        the given arrays (e.g. pinned host buffers) or new ones."""
        n = 3 * sum(s.natom for s in self.systems)
        x = np.zeros(n) if x is None else x
        v = np.zeros(n) if v is None else v
        self._check(self.lib.qgpu_get_coords_all(self.h, abi.ptr(x), abi.ptr(v)))
        return x, v

    # ----------------------------------------------------------- call points
    def make_pair_lists(self):
        self._check(self.lib.qgpu_build_lists(self.h))

    def pot_energy(self, traj: int = 0, terms: int = abi.QGPU_TERMS_ALL, want_forces: bool = True):
        s = self.systems[traj]
        d = np.zeros(3 * s.natom) if want_forces else None
        E = abi.Energies()
        EQ = (abi.QEnergy * max(s.nstates, 1))()
        self._check(self.lib.qgpu_forces(self.h, traj, terms, abi.ptr(d), C.byref(E), EQ))
        return d, E.as_dict(), [EQ[k].as_dict() for k in range(s.nstates)]

    def shake(self, traj: int, xx, x) -> tuple[np.ndarray, int]:
        xx = np.ascontiguousarray(xx, np.float64)
        out = np.ascontiguousarray(x, np.float64).copy()
        it = C.c_int32()
        self._check(self.lib.qgpu_shake(self.h, traj, abi.ptr(xx), abi.ptr(out), C.byref(it)))
        return out, it.value

    def temperature(self, traj: int = 0) -> np.ndarray:
        out = np.zeros(4)
        self._check(self.lib.qgpu_get_temperature(self.h, traj, abi.ptr(out)))
        return out

    def group_pairs(self, traj: int = 0) -> np.ndarray:
        n = C.c_int64()
        self._check(self.lib.qgpu_get_group_pairs(self.h, traj, None, 0, C.byref(n)))
        out = np.zeros((max(n.value, 1), 2), dtype=np.int32)
        self._check(self.lib.qgpu_get_group_pairs(self.h, traj, abi.ptr(out), n.value, C.byref(n)))
        return out[: n.value]

    def q_lists(self, traj: int = 0):
        """(solute atoms, water O atoms) on the Q-atom lists of the last list
        build (qgpu_get_q_lists), 0-based, ascending."""
        n = self.systems[traj].natom
        qp, qw = np.zeros(n, np.int32), np.zeros(n, np.int32)
        npp, nww = C.c_int64(), C.c_int64()
        self._check(self.lib.qgpu_get_q_lists(self.h, traj, abi.ptr(qp), n, C.byref(npp), abi.ptr(qw), n,
                                              C.byref(nww)))
        return qp[:npp.value].copy(), qw[:nww.value].copy()

    def shake_counts(self):
        """(molecule sweeps, constraint visits) of SHAKE since the last call
        (qgpu_shake_counts; the counters restart)."""
        sw, vi = C.c_int64(), C.c_int64()
        self._check(self.lib.qgpu_shake_counts(self.h, C.byref(sw), C.byref(vi)))
        return sw.value, vi.value

    def lrf(self, traj: int = 0) -> np.ndarray:
        out = np.zeros((len(self.systems[traj].cgp_first), 43))
        self._check(self.lib.qgpu_get_lrf(self.h, traj, abi.ptr(out)))
        return out

    # ---------------------------------------------------- energy files, FEP
    def ene_open(self, traj: int, path: str):
        """Attach a Q energy file to trajectory traj (qgpu_ene_open)."""
        self._check(self.lib.qgpu_ene_open(self.h, traj, path.encode()))

    def ene_close(self, traj: int):
        self._check(self.lib.qgpu_ene_close(self.h, traj))

    def fep_start(self, chain, kT: float, nskip: int = 0):
        """Start the device FEP sums over the window chain (trajectories in
        lambda order, qgpu_fep_start)."""
        c = np.ascontiguousarray(chain, dtype=np.int32)
        self._fep_n = len(c)
        self._check(self.lib.qgpu_fep_start(self.h, len(c), abi.ptr(c), kT, nskip))

    def fep_result(self):
        """(dgf, dgr, dG, stats[nwin, 7]) of qfep Part 1 from the device sums."""
        n = self._fep_n
        dgf, dgr, dg, st = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros((n, 7))
        self._check(self.lib.qgpu_fep_result(self.h, abi.ptr(dgf), abi.ptr(dgr), abi.ptr(dg), abi.ptr(st)))
        return dgf, dgr, dg, st

    def autotune(self) -> list:
        """Time the pair-kernel launch shapes and keep the fastest
        (qgpu_autotune); returns [lanes_water, min_blocks_water,
        lanes_solute, lanes_qw, unroll_water]."""
        t = np.zeros(5, dtype=np.int32)
        self._check(self.lib.qgpu_autotune(self.h, abi.ptr(t)))
        return [int(v) for v in t]

    def set_tuning(self, tuning):
        t = np.ascontiguousarray(tuning, dtype=np.int32)
        self._check(self.lib.qgpu_set_tuning(self.h, abi.ptr(t)))

    def set_step(self, istep: int):
        self._check(self.lib.qgpu_set_step(self.h, istep))

    def set_branches(self, n: int):
        """Independent trajectory groups of the replayed blocks (qgpu_set_branches)."""
        self._check(self.lib.qgpu_set_branches(self.h, n))

    def branches(self) -> int:
        return int(self.lib.qgpu_get_branches(self.h))

    def set_precision(self, mode: int):
        """QGPU_PRECISION_MIXED (default) or QGPU_PRECISION_FP64 for the MD
        step (see qgpu_set_precision)."""
        self._check(self.lib.qgpu_set_precision(self.h, mode))

    def enqueue(self, nsteps: int, ene_every: int = 0):
        """Queue nsteps of device work without waiting (see qgpu_enqueue)."""
        self._check(self.lib.qgpu_enqueue(self.h, nsteps, ene_every))

    def sync(self):
        self._check(self.lib.qgpu_sync(self.h))

    def stream(self) -> int:
        return int(self.lib.qgpu_stream(self.h) or 0)

    def profile(self, nsteps: int) -> dict:
        """Per-kernel (total ms, launches) over nsteps kernel-by-kernel steps."""
        cap = 64
        names = C.create_string_buffer(64 * cap)
        ms = np.zeros(cap)
        cnt = np.zeros(cap, dtype=np.int64)
        n = C.c_int32()
        self._check(self.lib.qgpu_profile(self.h, nsteps, names, abi.ptr(ms), abi.ptr(cnt), cap, C.byref(n)))
        raw = names.raw
        return {raw[64 * k:64 * (k + 1)].split(b"\0")[0].decode(): (float(ms[k]), int(cnt[k])) for k in range(n.value)}

    def run_rows(self, nsteps: int, ene_every: int, E, EQ, traj, step) -> int:
        """qgpu_run_rows: the energy records in preallocated arrays (E:
        Energies[cap], EQ: QEnergy[cap * MAX_STATES], traj/step: int32[cap]).
        Returns the number of rows the run produced."""
        n = C.c_int32()
        self._check(self.lib.qgpu_run_rows(self.h, nsteps, ene_every, C.cast(E, C.c_void_p), C.cast(EQ, C.c_void_p),
                                           abi.ptr(traj), abi.ptr(step), len(traj), C.byref(n)))
        return n.value

    def run(self, nsteps: int, ene_every: int = 0, collect: bool = True):
        """Run nsteps MD steps of every trajectory on the device.  Returns a
        list per trajectory of (step, E dict, [EQ dicts]) rows."""
        rows: list[list] = [[] for _ in range(self.ntraj)]

        def sink(user, traj, step, eq, ns, e):
            rows[traj].append((step, e.contents.as_dict(), [eq[k].as_dict() for k in range(ns)]))

        cb = abi.ENE_SINK(sink) if collect and ene_every > 0 else abi.ENE_SINK()
        self._check(self.lib.qgpu_run(self.h, nsteps, ene_every, cb, None))
        return rows
