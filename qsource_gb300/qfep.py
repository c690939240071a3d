"""qfep's free-energy analysis of Q energy files: FEP (Part 1) and the EVB
mapping (Parts 2 and 3, src/qfep.f90:416-835), through qgpu_qfep_evb.

The arguments mirror qfep's interactive input (src/qfep.f90:110-230): number
of states and of off-diagonal elements stored in the files, kT, points to
skip, calculation mode (gas), gap bins, minimum points per bin, alpha of
states 2.., Hij scaling or explicit couplings (i, j, A, mu, eta, r_xy0), and
the linear combination of states that defines the reaction coordinate.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi


def evb(paths, nstates: int, kT: float, *, noffd: int = 0, nskip: int = 0, gas: bool = False, nbins: int = 20,
        nmin: int = 1, alpha=None, scale_hij: float = 0.0, couplings=(), coeff=None, lib=None) -> dict:
    """paths: energy files in lambda order.  couplings: (i, j, A, mu, eta,
    r_xy0) tuples with 1-based states, used when noffd == 0.  coeff defaults
    to (-1, 1, 0, ...): the gap V_2 - V_1.

    Returns dict with part1 [nfiles, 3] (dGf, dGr, dG), gap (min, max),
    part2 [nfiles, nbins, 5 + nstates] (points, gap, dGg, c1, c2, dGv per
    state), part3 [nbins, 7] (points, gap, <dGg>, <dGg> - min, c1, c2, r_xy)
    and npts per file."""
    lib = lib or abi.load_library()
    P = abi.QfepParams()
    P.nstates, P.noffd, P.kT, P.nskip, P.gas, P.nbins, P.nmin = nstates, noffd, kT, nskip, int(gas), nbins, nmin
    for s, a in enumerate(alpha or []):
        P.alpha[s] = a
    P.scale_hij = scale_hij
    if len(couplings) > abi.QFEP_MAXCOUP:
        raise ValueError("too many couplings")
    P.ncoup = len(couplings)
    for c, (i, j, A, mu, eta, r0) in enumerate(couplings):
        P.coup_ij[2 * c], P.coup_ij[2 * c + 1] = i, j
        P.coup_A[c], P.coup_mu[c], P.coup_eta[c], P.coup_rxy0[c] = A, mu, eta, r0
    cf = list(coeff) if coeff is not None else [-1.0, 1.0] + [0.0] * (nstates - 2)
    for s, c in enumerate(cf):
        P.coeff[s] = c
    n = len(paths)
    arr = (C.c_char_p * n)(*[str(p).encode() for p in paths])
    part1 = np.zeros((n, 3))
    gap = np.zeros(2)
    part2 = np.zeros((n, nbins, abi.QFEP_P2))
    part3 = np.zeros((nbins, abi.QFEP_P3))
    npts = np.zeros(n, dtype=np.int32)
    rc = lib.qgpu_qfep_evb(n, arr, C.byref(P), abi.ptr(part1), abi.ptr(gap), abi.ptr(part2), abi.ptr(part3),
                           abi.ptr(npts))
    if rc != 0:
        raise RuntimeError(abi.last_error(lib))
    return {"part1": part1, "gap": gap, "part2": part2[:, :, :5 + nstates], "part3": part3, "npts": npts}
