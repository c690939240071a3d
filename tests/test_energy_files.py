"""Q energy files (.en) and the qfep free-energy restatement (no GPU).

* The library's writer (qgpu_enefile_write, host code) produces the record
  layout of put_ene (src/nrgy.f90:94-123) with the header of
  prep_sim_version (src/md.f90:17011-17015): checked byte by byte with an
  independent struct parse.
* The oracle's qfep Part 1 (src/qfep.f90:609-661) on such files equals the
  Zwanzig sums written out with numpy (1e-12 relative).
"""
import ctypes as C
import os
import struct

import numpy as np


def _frames(rng, nwin, npts, S=2):
    """Per window: npts frames of S states with random state totals."""
    lam = [(1.0 - w / (nwin - 1), w / (nwin - 1)) for w in range(nwin)]
    V = rng.normal(0.0, 2.0, size=(nwin, npts, S)) + np.array([0.0, 1.5])
    return lam, V


def _write(lib, path, lam, V, offd=None):
    from qsource_gb300.abi import QEnergy
    npts, S = V.shape
    rows = (QEnergy * (npts * S))()
    for p in range(npts):
        for s in range(S):
            q = rows[p * S + s]
            q.lambda_ = lam[s]
            q.total = V[p, s]
            q.q_bond, q.q_angle, q.qx_el, q.qw_vdw, q.restraint = 1.0 * s, 2.0, V[p, s] - 3.0, 3.0, 0.0
    if offd is None:
        rc = lib.qgpu_enefile_write(path.encode(), npts, S, rows, 0, None, None)
    else:
        ij, Hr = offd
        rc = lib.qgpu_enefile_write(path.encode(), npts, S, rows, len(ij) // 2, ij.ctypes.data_as(C.c_void_p),
                                    Hr.ctypes.data_as(C.c_void_p))
    assert rc == 0


def _records(path):
    out = []
    with open(path, "rb") as f:
        data = f.read()
    k = 0
    while k < len(data):
        n = struct.unpack_from("<i", data, k)[0]
        out.append(data[k + 4:k + 4 + n])
        assert struct.unpack_from("<i", data, k + 4 + n)[0] == n
        k += 8 + n
    return out


def test_energy_file_record_layout(engine_lib, tmp_path):
    rng = np.random.default_rng(5)
    lam, V = _frames(rng, 2, 3)
    ij = np.array([1, 2], dtype=np.int32)
    Hr = np.array([[20.0, 2.5], [19.0, 2.6], [18.0, 2.7]])
    path = str(tmp_path / "w0.en")
    _write(engine_lib, path, lam[0], V[0], offd=(ij, Hr))
    recs = _records(path)
    assert len(recs) == 1 + 3 * (2 + 1)
    canary, arrays, totresid, types, numres, resid, gcnum = struct.unpack_from("<7i", recs[0])
    assert (canary, arrays, totresid, types, numres, resid, gcnum) == (1337, 1, 1, 3, 1, -1, -1)
    assert len(recs[0]) == 7 * 4 + 80
    for p in range(3):
        for s in range(2):
            r = recs[1 + 3 * p + s]
            assert len(r) == 4 + 15 * 8
            i = struct.unpack_from("<i", r)[0]
            vals = struct.unpack_from("<15d", r, 4)
            assert i == s + 1 and vals[0] == lam[0][s] and vals[1] == V[0, p, s]
            assert vals[6] == V[0, p, s] - 3.0 and vals[13] == 3.0   # qx%el, qw%vdw
        od = recs[1 + 3 * p + 2]
        assert len(od) == 24 and struct.unpack_from("<2i2d", od) == (1, 2, Hr[p, 0], Hr[p, 1])


def test_qfep_restatement_matches_zwanzig(engine_lib, tmp_path):
    from oracle.oracle import qfep_fep
    rng = np.random.default_rng(7)
    nwin, npts, kT, nskip = 5, 40, 0.596163, 4
    lam, V = _frames(rng, nwin, npts)
    paths = []
    for w in range(nwin):
        p = str(tmp_path / f"w{w}.en")
        _write(engine_lib, p, lam[w], V[w])
        paths.append(p)
    dgf, dgr, dg, npt = qfep_fep(paths, 2, kT, nskip)
    assert list(npt) == [npts] * nwin
    L = np.array(lam)
    ref_f, ref_r = np.zeros(nwin), np.zeros(nwin)
    for w in range(nwin - 1):
        dv = V[w, nskip:] @ L[w + 1] - V[w, nskip:] @ L[w]
        ref_f[w] = -kT * np.log(np.mean(np.exp(-dv / kT)))
    for w in range(1, nwin):
        dv = V[w, nskip:] @ L[w - 1] - V[w, nskip:] @ L[w]
        ref_r[w] = -kT * np.log(np.mean(np.exp(-dv / kT)))
    ref_g = np.concatenate([[0.0], np.cumsum(0.5 * (ref_f[:-1] - ref_r[1:]))])
    assert np.allclose(dgf, ref_f, rtol=1e-12, atol=1e-12)
    assert np.allclose(dgr, ref_r, rtol=1e-12, atol=1e-12)
    assert np.allclose(dg, ref_g, rtol=1e-12, atol=1e-12)
