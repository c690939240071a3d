"""The metric's qualifier at production length: Delta-G of the 21-window chain
of the 18 A droplet (config 3's windows, lambda_A from 1 to 0 in steps of
0.05; the 8-atom Q chain discharged, its centre held at the droplet centre by
a sequence restraint of 5 kcal/(mol A^2) -- without it the neutral chain of
the discharged windows leaves the droplet within a few hundred picoseconds)
from the batched FP64-master engine:

  * against the FP64 oracle's own trajectories of every window over the
    first OR_STEPS steps from the same start: the engine's dG over the same
    steps agrees within 3 combined block-averaged standard errors (the two
    trajectories separate after about a picosecond, so they are compared as
    samples of the same ensemble);
  * against a run of the same systems 20 times longer from other initial
    velocities: within 3 combined block errors; the chain dG of each tenth of
    the long run is printed beside it.

(The metric's own comparison -- batched against the plain form, each window
alone -- is exact: a trajectory gives the same bits alone or in a batch,
tests/test_gpu_parity.py.)

Delta-G is qfep's Part 1 (src/qfep.f90:609-661, the restatement
oracle/qfep_ref.py) over the recorded frames after the first 10 %; the
standard error of a chain dG comes from NBLK blocks of consecutive frames
(dG of each block, their spread / sqrt(NBLK)).  The reference ships no golden
dG: this pins dG by the oracle's dynamics and the qfep restatement.

Long: a few minutes of GPU and about ten minutes of host-core time.  It runs
when QGPU_LONG=1 is set; otherwise it is skipped."""
import multiprocessing as mp
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NWIN = 21
PROD_STEPS, LONG_FACTOR, OR_STEPS, EVERY, EVERY_LONG, NBLK = 50_000, 20, 10_000, 10, 50, 10
KT = 0.001986 * 300.0


def _chain(velocity_seed=None):
    """The 21 windows; velocity_seed draws other Maxwell velocities at 300 K
    for the same systems."""
    from qsource_gb300 import synth
    out = []
    for w in range(NWIN):
        la = 1.0 - w / (NWIN - 1)
        s = synth.config(1, window=w, lambdas=(la, 1.0 - la), solute_restraint=5.0)
        if velocity_seed is not None:
            rng = np.random.default_rng(velocity_seed + w)
            sd = np.sqrt(0.001986 * 300.0 / np.asarray(s.mass)[np.asarray(s.iac)])
            s.v = (rng.normal(size=(s.natom, 3)) * sd[:, None]).reshape(-1)
        out.append(s)
    return out


def dg_chain(windows, nskip_frac=0.1, blocks_out=None):
    """Chain dG (qfep Part 1) and its block standard error from windows given
    as (lambdas, frames); blocks_out receives the dG of each block."""
    from oracle import qfep_ref
    n = min(len(f) for _, f in windows)
    skip = int(nskip_frac * n)
    dg = qfep_ref.evb_windows(windows, 2, KT, nskip=skip)["part1"][-1, 2]
    use = n - skip
    b = use // NBLK
    blocks = []
    for k in range(NBLK):
        sub = [(lam, f[skip + k * b:skip + (k + 1) * b]) for lam, f in windows]
        blocks.append(qfep_ref.evb_windows(sub, 2, KT, nskip=0)["part1"][-1, 2])
    if blocks_out is not None:
        blocks_out.extend(float(b) for b in blocks)
    return float(dg), float(np.std(blocks, ddof=1) / np.sqrt(NBLK))


def _engine_windows(systems, nsteps, tmp, tag, every=EVERY):
    from oracle import qfep_ref
    from qsource_gb300.engine import Engine
    e = Engine(systems)
    paths = [os.path.join(tmp, f"{tag}{w:02d}.en") for w in range(len(systems))]
    for w, p in enumerate(paths):
        e.ene_open(w, p)
    e.run(nsteps, ene_every=every, collect=False)
    for w in range(len(systems)):
        e.ene_close(w)
    e.close()
    return [qfep_ref.read_en(p, 2, 0) for p in paths]


@pytest.mark.skipif(os.environ.get("QGPU_LONG") != "1", reason="long run: set QGPU_LONG=1")
def test_dg_production_against_long_run_and_oracle(engine_lib, tmp_path):
    from oracle.oracle import md_frames
    prod = _chain()
    # the oracle's trajectories on the host cores meanwhile (spawned workers)
    with mp.get_context("spawn").Pool(min(NWIN, os.cpu_count() or 1)) as pool:
        pending = pool.starmap_async(md_frames, [(s, OR_STEPS, EVERY, []) for s in prod])
        w_prod = _engine_windows(prod, PROD_STEPS, str(tmp_path), "p")
        w_long = _engine_windows(_chain(velocity_seed=7919), PROD_STEPS * LONG_FACTOR, str(tmp_path), "l",
                                 EVERY_LONG)
        w_or = pending.get(timeout=7200)
    dg_p, se_p = dg_chain(w_prod)
    long_blocks = []
    dg_l, se_l = dg_chain(w_long, blocks_out=long_blocks)
    # the engine over the oracle's span, from the same start
    w_short = [(lam, f[:len(fo)]) for (lam, f), (_, fo) in zip(w_prod, w_or)]
    dg_s, se_s = dg_chain(w_short)
    dg_o, se_o = dg_chain(w_or)
    print(f"dG chain: production {PROD_STEPS} steps {dg_p:.3f} +- {se_p:.3f}; long {PROD_STEPS * LONG_FACTOR} steps "
          f"{dg_l:.3f} +- {se_l:.3f}; first {OR_STEPS} steps: engine {dg_s:.3f} +- {se_s:.3f}, "
          f"oracle {dg_o:.3f} +- {se_o:.3f} kcal/mol")
    print("dG long-run blocks:", " ".join(f"{b:.2f}" for b in long_blocks))
    assert abs(dg_s - dg_o) <= 3.0 * np.hypot(se_s, se_o)
    assert abs(dg_p - dg_l) <= 3.0 * np.hypot(se_p, se_l)
