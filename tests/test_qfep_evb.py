"""qfep's EVB mapping (Parts 1-3) on energy files, host code (no GPU).

qgpu_qfep_evb against the line-by-line numpy restatement of src/qfep.f90
(oracle/qfep_ref.py, its own reader of the files) on synthetic two- and
three-state EVB windows written by qgpu_enefile_write: diabatic parabolas
along a sampled coordinate, the coupling in the file (scaled) or given as
A exp(-mu (r - r0)) exp(-eta (r - r0)^2) of the file's distance, alpha
shifts, skipped points, the gas mode and qfep's normalisation of Part 3
(minimum over every bin, empty ones included).  Agreement 1e-9 kcal/mol.

Parity unpinned by reference data: the reference ships no EVB mapping output
(its mapping test lacks the restart files), so Parts 2-3 are pinned by the
restatement only."""
import ctypes as C

import numpy as np
import pytest

KT = 0.5925


def _windows(lib, tmp_path, nstates, nwin=11, npts=400, seed=3):
    from qsource_gb300.abi import QEnergy
    rng = np.random.default_rng(seed)
    paths = []
    for w in range(nwin):
        lw = w / (nwin - 1)
        lam = [1.0 - lw, lw] if nstates == 2 else [max(0.0, 1 - 2 * lw), 1 - abs(1 - 2 * lw), max(0.0, 2 * lw - 1)]
        x = rng.normal(lw, 0.12, npts)
        rows = (QEnergy * (npts * nstates))()
        # one off-diagonal entry per coupling of the case: (1,2) and (2,3)
        noff = nstates - 1
        ij = np.array([1, 2, 2, 3][:2 * noff], dtype=np.int32)
        Hr = np.zeros((npts, noff, 2))
        for p in range(npts):
            E = [80.0 * x[p] ** 2, 80.0 * (x[p] - 1.0) ** 2 - 6.0, 80.0 * (x[p] - 0.5) ** 2 + 3.0][:nstates]
            r = 2.0 + 0.6 * x[p] + rng.normal(0, 0.02)
            for c in range(noff):
                Hr[p, c] = [30.0 * np.exp(-0.8 * (r - 2.0)) / (c + 1), r + c]
            for s in range(nstates):
                q = rows[p * nstates + s]
                q.lambda_ = lam[s]
                q.total = E[s]
                q.q_bond, q.q_angle, q.q_torsion, q.q_improper = 0.3 * E[s], 1.0 + s, 0.5, 0.25
                q.qq_el, q.qq_vdw, q.restraint = 0.2 * E[s], -1.5, 0.1 * s
                q.qx_el, q.qw_vdw = E[s] - 5.0, 2.0
        path = str(tmp_path / f"evb{nstates}_{w:02d}.en")
        assert lib.qgpu_enefile_write(path.encode(), npts, nstates, rows, noff, ij.ctypes.data_as(C.c_void_p),
                                      Hr.ctypes.data_as(C.c_void_p)) == 0
        paths.append(path)
    return paths


CASES = {
    "file_hij_scaled": (2, dict(noffd=1, scale_hij=1.3, alpha=[0.0, 4.0], nskip=20, nbins=24, nmin=8)),
    "explicit_coupling_gas": (2, dict(noffd=0, couplings=[(1, 2, 25.0, 0.7, 0.05, 2.1)], gas=True, nbins=16,
                                      nmin=5)),
    "three_states": (3, dict(noffd=0, couplings=[(1, 2, 20.0, 0.5, 0.0, 2.0), (3, 2, 12.0, 0.3, 0.1, 2.2)],
                             alpha=[0.0, 2.0, -1.0], coeff=[-1.0, 0.0, 1.0], nbins=20, nmin=4, nskip=5)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_evb_mapping_matches_qfep_restatement(engine_lib, tmp_path, name):
    from oracle import qfep_ref
    from qsource_gb300 import qfep
    S, kw = CASES[name]
    paths = _windows(engine_lib, tmp_path, S)
    got = qfep.evb(paths, S, KT, lib=engine_lib, **kw)
    ref = qfep_ref.evb(paths, S, KT, **kw)
    np.testing.assert_array_equal(got["npts"], ref["npts"])
    for key in ("part1", "gap", "part2", "part3"):
        np.testing.assert_allclose(got[key], ref[key], rtol=0, atol=1e-9, err_msg=key)
    p2, p3 = got["part2"], got["part3"]
    assert (p3[:, 0] >= kw["nmin"]).sum() >= kw["nbins"] // 2          # the windows cover the gap range
    on = p3[:, 0] >= kw["nmin"]
    assert np.isclose(p3[on, 3].min(), p3[on, 2].min() - min(0.0, p3[on, 2].min()))   # qfep's min includes empty bins
    if S == 2:
        c = p2[p2[:, :, 0] >= kw["nmin"]]
        np.testing.assert_allclose(c[:, 3] + c[:, 4], 1.0, atol=1e-12)
        # the ground state lies below both diabatic curves in every bin
        assert np.all(c[:, 2] <= np.minimum(c[:, 5], c[:, 6]) + 1e-9)


def test_evb_rejects_bad_input(engine_lib, tmp_path):
    from qsource_gb300 import qfep
    paths = _windows(engine_lib, tmp_path, 2, nwin=2, npts=10)
    with pytest.raises(RuntimeError):
        qfep.evb(paths[:1], 2, KT, lib=engine_lib)                       # one file: no Parts 1-3
    with pytest.raises(RuntimeError):
        qfep.evb(paths, 2, KT, nskip=10, lib=engine_lib)                 # nothing left after skipping
    with pytest.raises(RuntimeError):
        qfep.evb(paths, 3, KT, noffd=1, scale_hij=1.0, lib=engine_lib)   # scaling is for two states
    with pytest.raises(RuntimeError):
        qfep.evb([paths[0], str(tmp_path / "missing.en")], 2, KT, lib=engine_lib)
