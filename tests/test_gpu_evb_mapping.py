"""Config 4's EVB mapping: the 35 A sphere with the 3,000-atom chain and a
30-atom Q region in 4 EVB states (charge sets N(0, 0.5), constant
off-diagonal Hij = 20 kcal/mol between every pair of states), run as 51
batched lambda windows in one engine handle (lambda_1 from 1 to 0 in steps of
0.02 with lambda_2 = 1 - lambda_1, the window spacing of the reference's
mapping protocol), FP64-master step, energy files written by the engine.

  * qfep Parts 1-3 (src/qfep.f90:416-835) on the engine's 51 files: the
    engine's host code (qgpu_qfep_evb) equals the numpy restatement of qfep
    to 1e-9 kcal/mol at 4 states (EVB ground state of the 4x4 Hamiltonian).
  * The same mapping on the FP64 oracle's own trajectories of the 51 windows
    (same start, same steps; run on the host cores): the energy gaps of
    every frame, the gap histogram of every window (Part 2 bin counts) and
    the free-energy profiles (Parts 1-3) agree within the stated tolerances.
    Over 50 steps the engine's and the oracle's trajectories stay within
    about 1e-4 kcal/mol of each other, far below the 0.1 kcal/mol bar.
Parity unpinned by reference data: the reference ships no EVB mapping output
for this system, so the mapping's arithmetic is pinned by the restatement of
qfep and the dynamics by the oracle."""
import copy
import multiprocessing as mp
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NWIN, NSTEPS, EVERY = 51, 50, 5
KT = 0.001986 * 300.0
COUPLINGS = [(i + 1, j + 1, 20.0, 0.0, 0.0, 0.0) for i in range(4) for j in range(i + 1, 4)]
QFEP = dict(nskip=0, nbins=12, nmin=2)


def _windows():
    from qsource_gb300 import synth
    base = synth.config(4)
    out = []
    for w in range(NWIN):
        s = copy.copy(base)
        s._keep = []       # each window's descriptor keeps its own arrays alive
        la = 1.0 - w / (NWIN - 1)
        s.lambdas = [la, 1.0 - la, 0.0, 0.0] + [0.0] * (len(base.lambdas) - 4)
        out.append(s)
    return out


def test_cfg4_51_window_mapping(engine_lib, tmp_path):
    from oracle import qfep_ref
    from oracle.oracle import md_frames
    from qsource_gb300 import qfep
    from qsource_gb300.engine import Engine
    systems = _windows()
    # the oracle's trajectories on the host cores (spawned workers: no CUDA state)
    with mp.get_context("spawn").Pool(min(NWIN, os.cpu_count() or 1)) as pool:
        pending = pool.starmap_async(md_frames, [(s, NSTEPS, EVERY, [c[:3] for c in COUPLINGS]) for s in systems])
        e = Engine(systems)
        paths = [str(tmp_path / f"w{w:02d}.en") for w in range(NWIN)]
        for w, p in enumerate(paths):
            e.ene_open(w, p)
        e.run(NSTEPS, ene_every=EVERY, collect=False)
        for w in range(NWIN):
            e.ene_close(w)
        oracle_windows = pending.get(timeout=1800)
    # engine files: the library's qfep against the restatement
    got = qfep.evb(paths, 4, KT, lib=engine_lib, couplings=COUPLINGS, **QFEP)
    ref = qfep_ref.evb(paths, 4, KT, couplings=COUPLINGS, **QFEP)
    for key in ("part1", "gap", "part2", "part3"):
        np.testing.assert_allclose(got[key], ref[key], rtol=0, atol=1e-9, err_msg=key)
    assert list(ref["npts"]) == [NSTEPS // EVERY - 1] * NWIN
    # engine trajectories against the oracle's
    eng_windows = [qfep_ref.read_en(p, 4, len(COUPLINGS)) for p in paths]
    worst_gap = 0.0
    for (le, fe), (lo, fo) in zip(eng_windows, oracle_windows):
        assert np.allclose(le, lo, atol=1e-12)
        for (Ee, _), (Eo, _) in zip(fe, fo):
            worst_gap = max(worst_gap, abs((Ee[1] - Ee[0]) - (Eo[1] - Eo[0])))
    ora = qfep_ref.evb_windows(oracle_windows, 4, KT, couplings=COUPLINGS, **QFEP)
    print(f"config 4 mapping: worst |gap difference| {worst_gap:.2e} kcal/mol over {NWIN} x {NSTEPS // EVERY - 1} "
          f"frames; dG(chain) engine {ref['part1'][-1, 2]:.4f} oracle {ora['part1'][-1, 2]:.4f}")
    assert worst_gap < 0.01
    np.testing.assert_allclose(ref["part1"], ora["part1"], rtol=0, atol=0.01)
    # histograms: a frame may move to a neighbouring bin only if its gap lies
    # within the gap difference of a bin edge; the bin layout itself follows
    # the extreme gaps
    np.testing.assert_allclose(ref["gap"], ora["gap"], rtol=0, atol=0.01)
    counts_e, counts_o = ref["part2"][:, :, 0], ora["part2"][:, :, 0]
    assert np.abs(counts_e - counts_o).sum() <= 2 * NWIN * 0.1 * (NSTEPS // EVERY)
    both = (ref["part3"][:, 0] >= QFEP["nmin"]) & (ora["part3"][:, 0] >= QFEP["nmin"])
    assert both.sum() >= 6
    np.testing.assert_allclose(ref["part3"][both, 2], ora["part3"][both, 2], rtol=0, atol=0.05)
