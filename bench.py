"""Benchmark of the GB300 qdyn hot-path engine on the lambda-window batch.

Workload (one "step" = one MD step of every trajectory of the batch): the
lambda-window batch of 21 windows (lambda_A = 1 ... 0 in steps of 0.05) of the
18 A TIP3P droplet with an 8-atom, 2-state Q region, plus 11 uneven replicas
(20/25/30 A spheres with 500- to 2,000-atom solutes), 32 trajectories in one
engine handle; Berendsen 300 K, 1 fs, SHAKE on waters, lists + LRF every 10
steps, each 10-step block replayed from one CUDA graph.  Synthetic seeded
systems (qsource_gb300.synth), not a public data set.

Precision: the FP64-master step (QGPU_PRECISION_FP64: FP64 x, v, leap-frog,
SHAKE and temperatures; FP32 pair terms; int64 fixed-point sums) unless
--precision mixed.

Printed: one JSON line (rank 0).  `value` = aggregate ns/day from CUDA events
on the engine's stream around the timed 10-step blocks (L2 flushed with a
256 MB write before each block); `e2e` = the same through the public API with
host buffers (coordinates and velocities uploaded from pinned memory and read
back, energies read back every block, a .en energy file written per
trajectory and the device FEP sums of the 21-window chain accumulated);
`mixed_form` = the same timed loop with the mixed-precision step (float
master state), a secondary figure with its own dtype; `plain_form` = the same
trajectories run one at a time, each alone in its own autotuned handle (the
unbatched GPU form), and `batched_over_plain` = value / plain_form.
--impl reference times the FP64 CPU restatement of the reference (oracle/) on
all host cores instead.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "agg. ns/day (λ-window batch, 1 GB300) at ≤0.1 kcal/mol ΔG vs plain-form GPU"
NB = 10
FS_PER_STEP = 1.0
# what each step form computes in which arithmetic
DTYPE = {
    "fp64": ("f64 master x/v, thermostat + leap-frog update, SHAKE and temperature; f64 list cut-off test and "
             "recorded-step per-state Q energies; f32 pair/LRF terms from double-float coordinate differences; int64 "
             "fixed-point force and energy sums"),
    "mixed": ("double-float (~48-bit) master positions, f32 velocities, f32 3-site-water SHAKE and temperature, f32 "
              "pair/bonded terms on unrecorded steps; f64 list cut-off test and recorded-step energies; int64 "
              "fixed-point sums"),
}
KT_300 = 0.001986 * 300.0   # Boltz * T (src/md.f90:54), the FEP sums' kT
WORKLOAD = ("lambda-window batch: 21 windows of the 18 A droplet (8 Q atoms, 2 states) + 11 uneven replicas "
            "(20/25/30 A spheres, 500-2000-atom solutes) = 32 trajectories")


# ------------------------------------------------------------ CPU arm
NTRAJ = 32


def _cpu_traj(args):
    """One trajectory of the batch on one host core with the FP64 C
    restatement of the reference: `warm` untimed steps, then `nsteps` timed
    steps (lists every 10 steps, Berendsen leap-frog, SHAKE).  Returns the
    timed seconds."""
    i, warm, nsteps = args
    sys.path.insert(0, ROOT)
    from qsource_gb300 import synth
    from oracle.oracle import Oracle
    o = Oracle(synth.lambda_batch_member(i))
    o.temperature()
    if warm:
        o.md_run(warm)
    t0 = time.perf_counter()
    rc, _, _, _ = o.md_run(nsteps)
    dt = time.perf_counter() - t0
    if rc:
        raise RuntimeError(f"oracle trajectory {i}: status {rc}")
    return i, dt


def _makespan(times, cores):
    """Wall time of running the given per-trajectory times on `cores` cores,
    longest first, each trajectory on the first free core."""
    free = [0.0] * cores
    for t in sorted(times, reverse=True):
        k = free.index(min(free))
        free[k] += t
    return max(free)


def cpu_pool():
    """Process pool over every host core; started with spawn before any CUDA
    call of the parent process."""
    return mp.get_context("spawn").Pool(os.cpu_count() or 1)


def cpu_baseline(pool, nsteps: int, warm: int = 0):
    """Aggregate ns/day of the 32-trajectory batch on the host cores: every
    trajectory is timed on its own core (all cores busy at once); the batch
    wall time is the makespan of those times on the pool's cores."""
    cores = pool._processes
    jobs = [(i, warm, nsteps) for i in range(NTRAJ)]
    # longest trajectories (the replicas) first
    jobs.sort(key=lambda j: -j[0])
    t0 = time.perf_counter()
    res = dict(pool.map(_cpu_traj, jobs, chunksize=1))
    wall = time.perf_counter() - t0
    times = [res[i] for i in range(NTRAJ)]
    span = _makespan(times, cores)
    batch_step = span / nsteps
    nsday = NTRAJ * FS_PER_STEP * 1e-6 * 86400.0 / batch_step
    sample = (f"oracle (FP64 C restatement of the reference loops) on {cores} host cores, one trajectory per core: "
              f"all {NTRAJ} trajectories of the batch, {warm} untimed + {nsteps} timed Berendsen/SHAKE steps each "
              f"(lists every {NB} steps); batch step = makespan of the per-trajectory times on {cores} cores "
              f"({span:.2f} s for {nsteps} steps; single-core sum {sum(times):.2f} s; pool wall incl. set-up "
              f"{wall:.1f} s)")
    return {"value": round(nsday, 4), "unit": "ns/day", "cores": cores, "kind": "port", "sample": sample,
            "ms_per_batch_step": batch_step * 1e3, "single_core_ms_per_batch_step": 1e3 * sum(times) / nsteps}


# --------------------------------------------------------- clocks
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        dev = os.environ.get("LOCAL_RANK", "0")
        rows = [r for r in self.rows if len(r) >= 9 and r[0] == dev] or [r for r in self.rows if len(r) >= 9]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "").isdigit())
        mx = max((float(r[2]) for r in rows if r[2].replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------- work counts
def work_counts(engine):
    """Algorithmic work of one list build and one step, from the engine's
    own lists: water pairs, solute-water / solute-solute atom pairs, LRF
    atom-centre updates, Q-water pairs."""
    import numpy as np
    tot = {"ww_pairs": 0, "pw_atom_pairs": 0, "pp_atom_pairs": 0, "lrf_updates": 0, "qw_pair_states": 0,
           "qw_qwaters": 0, "nstates_qw": 0}
    for t, s in enumerate(engine.systems):
        gp = engine.group_pairs(t)
        ncs = s.ncgp_solute
        G = len(s.cgp_first)
        isq = np.asarray(s.iqatom) >= 0
        nonq = np.array([int((~isq[s.cgpatom[s.cgp_first[g]:s.cgp_last[g] + 1]]).sum()) for g in range(G)])
        w1, w2 = gp[:, 0] >= ncs, gp[:, 1] >= ncs
        tot["ww_pairs"] += int(np.sum(w1 & w2))
        pw = w1 ^ w2
        sg = np.where(w1[pw], gp[pw, 1], gp[pw, 0])
        tot["pw_atom_pairs"] += int(3 * nonq[sg].sum())
        pp = ~(w1 | w2)
        tot["pp_atom_pairs"] += int((nonq[gp[pp, 0]] * nonq[gp[pp, 1]]).sum())
        excl = np.asarray(s.excl)[np.asarray(s.cgp_switch)].astype(bool)
        live = ~excl
        src = int(nonq[live].sum())
        near = np.zeros(G, dtype=np.int64)
        np.add.at(near, gp[:, 0], nonq[gp[:, 1]])
        np.add.at(near, gp[:, 1], nonq[gp[:, 0]])
        far = (src - near - nonq)[live]
        tot["lrf_updates"] += int(far.sum())
        tot["qw_qwaters"] += s.nqat * s.nwat
        tot["qw_pair_states"] += s.nqat * s.nwat * s.nstates
    return tot


def kernel_flops(name, wc):
    """Reference-convention flop counts per launch (FMA = 2): water-water
    molecule pair 228, LJ+Coulomb atom pair 36 (pw pairs split half/half
    between the water and solute kernels, pp pairs counted once), LRF
    atom-centre update 190, Q-water (Q atom, water) 3*17 + S*(3*6 + 10);
    the FP64 update: 40 per SHAKE constraint visit (the visits counted on the
    device during the profiled steps) and 27 per atom (thermostat kick 3,
    drift 2, v = (x - xx)/dt 2 per component; kinetic energy 6)."""
    if name == "k_update_d":
        return 40.0 * wc["shake_visits_per_step"] + 27.0 * wc["atoms"]
    if name == "k_nb_water":
        return 228.0 * wc["ww_pairs"] + 0.5 * 36.0 * wc["pw_atom_pairs"]
    if name == "k_nb_solute":
        return 36.0 * wc["pp_atom_pairs"] + 0.5 * 36.0 * wc["pw_atom_pairs"]
    if name == "k_scan":
        return 190.0 * wc["lrf_updates"]
    if name == "k_qw":
        return 51.0 * wc["qw_qwaters"] + 28.0 * wc["qw_pair_states"]
    return None


def plain_form(systems, flush, nblk: int, world: int, precision: str, tune: bool) -> dict:
    """The same trajectories on the same GPU kernels, one trajectory per
    handle and one after another (the uniform-window form without batching):
    each trajectory gets its own handle (launch shapes from the autotuner,
    as the batched handle's, unless tune is False), the same step precision,
    one untimed block, then nblk timed 10-step graph replays with the L2
    flushed before each.  Aggregate ns/day = all simulated time / the summed
    device time, the throughput of running the windows one by one."""
    import torch
    from qsource_gb300.abi import PRECISION
    from qsource_gb300.engine import Engine
    ms_total = 0.0
    per = []
    for s in systems:
        e = Engine([s])
        if tune:
            e.autotune()
        e.set_precision(PRECISION[precision])
        e.enqueue(NB, 0)
        e.sync()
        ext = torch.cuda.ExternalStream(e.stream())
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nblk)]
        torch.cuda.synchronize()
        with torch.cuda.stream(ext):
            for b in range(nblk):
                flush.fill_(float(b))
                ev[b][0].record(ext)
                e.enqueue(NB, NB)
                ev[b][1].record(ext)
        e.sync()
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in ev)
        ms_total += ms
        per.append(ms / (nblk * NB))
        e.close()
    value = aggregate_ns_per_day(world, len(systems), nblk * NB, ms_total)
    return {"value": round(value, 3), "unit": "ns/day",
            "ms_per_step_min": round(min(per), 5), "ms_per_step_max": round(max(per), 5),
            "how": f"each of the {len(systems)} trajectories alone in its own handle "
                   f"({'autotuned' if tune else 'default'} launch shapes, {precision} step), "
                   f"one after another: 1 untimed + {nblk} timed 10-step CUDA-graph blocks each, L2 flushed "
                   f"before every block; aggregate = simulated ns / summed device time"}


# ------------------------------------------------------------- main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=20, help="timed oracle steps of the CPU baseline")
    ap.add_argument("--ref-max-steps", type=int, default=100, help="cap on the reference arm's timed steps")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--no-tune", action="store_true", help="default launch shapes instead of the autotuner's")
    ap.add_argument("--tuning", default=None,
                    help="fixed launch shapes lanes_water,min_blocks_water,lanes_solute,lanes_qw,unroll_water "
                         "instead of the autotuner's (profiling runs: the autotuner's timings mean nothing "
                         "under a profiler that serialises kernels)")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"],
                    help="MD step precision of the headline (qgpu_set_precision): FP64 master / double-float master")
    ap.add_argument("--no-mixed", action="store_true", help="skip timing the mixed-precision form")
    ap.add_argument("--branches", type=int, default=0,
                    help="independent trajectory groups of the replayed blocks (qgpu_set_branches; 0: library default)")
    ap.add_argument("--no-plain", action="store_true", help="skip the one-trajectory-at-a-time GPU form")
    ap.add_argument("--plain-blocks", type=int, default=20, help="timed 10-step blocks per trajectory, plain form")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    steps = max(NB, int(math.ceil(args.steps / NB)) * NB)
    # warm-up in whole 10-step blocks, so that the timed blocks start at a list
    # update and replay the block graphs (a block that starts between list
    # updates runs step by step)
    warm = max(NB, int(math.ceil(max(3, args.warmup) / NB)) * NB)

    if args.impl == "reference":
        if rank != 0:
            return
        # the whole K-step run of the batch, capped so that it ends in minutes
        ksteps = min(steps, args.ref_max_steps)
        with cpu_pool() as pool:
            base = cpu_baseline(pool, ksteps, warm=min(warm, NB))
        out = {"metric": METRIC, "value": base["value"], "unit": "ns/day", "impl": "reference", "n_gpus": args.gpus,
               "steps": ksteps, "warmup": min(warm, NB), "ms_per_step": round(base["ms_per_batch_step"], 3),
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
               "data": "synthetic (seeded water spheres, random-init)",
               "config": {"workload": WORKLOAD, "trajectories": NTRAJ, "dt_fs": FS_PER_STEP, "nbcycle": NB,
                          "parallelism": f"host cores ({base['cores']}), one trajectory per core"},
               "cpu_baseline": {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")},
               "e2e": {"value": base["value"], "unit": "ns/day", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return

    # the CPU-baseline pool is started before the first CUDA call
    pool = cpu_pool() if rank == 0 and not args.no_cpu else None
    import numpy as np
    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from qsource_gb300 import synth
    from qsource_gb300.engine import Engine

    # weak scaling: every rank runs its own batch of independent replicas
    # (same recipe, own seeds); no data-path collective
    systems = synth.lambda_batch(rank=rank)
    ntraj = len(systems)
    natoms = sum(s.natom for s in systems)
    eng = Engine(systems)
    if args.tuning:
        tuning = [int(v) for v in args.tuning.split(",")]
        eng.set_tuning(tuning)
    else:
        tuning = eng.autotune() if not args.no_tune else None
    from qsource_gb300.abi import PRECISION
    eng.set_precision(PRECISION[args.precision])
    if args.branches:
        eng.set_branches(args.branches)
    eng.enqueue(warm, 0)
    eng.sync()

    ext = torch.cuda.ExternalStream(eng.stream())
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    nblk = steps // NB
    ms, launches, clk = timed_blocks(eng, ext, flush, nblk, dist)
    ns_per_day = aggregate_ns_per_day(world, ntraj, steps, ms)

    # --- end to end through the public API with host buffers: per block the
    # coordinates and velocities of the whole batch go up from pinned memory,
    # the block runs with an energy sink, and x, v come back
    n3 = 3 * natoms
    xs = torch.empty(n3, dtype=torch.float64).pin_memory().numpy()
    vs = torch.empty(n3, dtype=torch.float64).pin_memory().numpy()
    eng.coords_all(xs, vs)
    e2e_blocks = max(2, min(nblk // 2, 100))
    from qsource_gb300 import abi
    cap = 4 * ntraj
    E_rows, EQ_rows = (abi.Energies * cap)(), (abi.QEnergy * (cap * abi.MAX_STATES))()
    tr_rows, st_rows = np.zeros(cap, np.int32), np.zeros(cap, np.int32)
    # the metric's Delta-G machinery runs inside the timed region: one .en file
    # per trajectory (qdyn's energy output, written by the host sink) and the
    # device's qfep Part 1 sums over the 21-window chain of the droplet
    import tempfile
    endir = tempfile.mkdtemp(prefix="qgpu_bench_en_")
    nwin = 21
    eng.fep_start(list(range(nwin)), KT_300)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for t in range(ntraj):
        eng.ene_open(t, os.path.join(endir, f"traj{t:02d}.en"))
    nrows = 0
    for b in range(e2e_blocks):
        eng.set_coords_all(xs, vs)
        nrows += eng.run_rows(NB, NB, E_rows, EQ_rows, tr_rows, st_rows)
        eng.coords_all(xs, vs)
    for t in range(ntraj):
        eng.ene_close(t)
    if nrows != ntraj * e2e_blocks:
        raise RuntimeError(f"e2e: {nrows} energy records for {e2e_blocks} blocks of {ntraj} trajectories")
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    fep_frames = int(eng.fep_result()[3][0, 0])
    en_bytes = sum(os.path.getsize(os.path.join(endir, f)) for f in os.listdir(endir))
    for f in os.listdir(endir):
        os.remove(os.path.join(endir, f))
    os.rmdir(endir)
    e2e = world * ntraj * e2e_blocks * NB * FS_PER_STEP * 1e-6 * 86400.0 / e2e_s
    h2d = sum(2 * 3 * s.natom * 8 for s in systems) / NB
    d2h = (sum(2 * 3 * s.natom * 8 for s in systems) + ntraj * (29 + 15 * 4) * 8) / NB

    # --- roofline of the dominant kernel
    eng.shake_counts()                      # restart the device's SHAKE counters
    prof = eng.profile(2 * NB)
    sweeps, visits = eng.shake_counts()
    wc = work_counts(eng)
    wc["shake_visits_per_step"] = visits / (2 * NB)
    wc["shake_sweeps_per_water_step"] = sweeps / (2 * NB) / max(1, sum(s.nwat for s in systems))
    wc["atoms"] = natoms
    peaks = {"fp32": ctypes_peak(eng, "qgpu_fp32_peak"), "fp64": ctypes_peak(eng, "qgpu_fp64_peak")}
    peak_src = {"fp32": "measured in this run: FP32 FMA-chain kernel over all SMs (qgpu_fp32_peak)",
                "fp64": "measured in this run: FP64 DFMA-chain kernel over all SMs (qgpu_fp64_peak)"}

    def bound_of(kname):
        return "fp64" if kname == "k_update_d" else "fp32"
    share = {k: round(v[0] / sum(x[0] for x in prof.values()), 4) for k, v in prof.items()}
    us_per_step = {k: round(1e3 * v[0] / (2 * NB), 2) for k, v in prof.items()}
    # every kernel with an algorithmic count: its own roofline fraction
    per_kernel = {}
    for kname, (kms_k, kcnt_k) in prof.items():
        fk = kernel_flops(kname, wc)
        if fk is not None and kcnt_k:
            ach = fk / (kms_k / kcnt_k * 1e-3) / 1e12
            per_kernel[kname] = {"bound": bound_of(kname), "achieved_tflops": round(ach, 4),
                                 "frac": round(ach / peaks[bound_of(kname)], 4),
                                 "us_per_launch": round(1e3 * kms_k / kcnt_k, 2)}
    # the dominant kernel by time among those with an algorithmic count
    name, (kms, kcnt) = max(((k, v) for k, v in prof.items() if kernel_flops(k, wc) is not None),
                            key=lambda kv: kv[1][0])
    fl = kernel_flops(name, wc)
    achieved = fl / (kms / kcnt * 1e-3) / 1e12
    bnd = bound_of(name)
    roof = {"bound": bnd, "kernel": name, "achieved": round(achieved, 4), "peak": round(peaks[bnd], 3),
            "unit": "TFLOP/s", "frac": round(achieved / peaks[bnd], 4), "traffic": committed_traffic(name),
            "peak_source": peak_src[bnd], "avg_launch_ms": round(kms / kcnt, 5), "flops_per_launch": fl,
            "share_of_step_kernels": share.get(name)}
    mixed = None
    if not args.no_mixed and args.precision != "mixed":
        eng.set_precision(PRECISION["mixed"])
        eng.enqueue(NB, 0)
        eng.sync()
        mblk = min(nblk, 100)
        mms, _, _ = timed_blocks(eng, ext, flush, mblk, dist)
        mixed = {"value": round(aggregate_ns_per_day(world, ntraj, mblk * NB, mms), 3), "unit": "ns/day",
                 "ms_per_step": round(mms / (mblk * NB), 5), "steps": mblk * NB, "dtype": DTYPE["mixed"],
                 "how": "the same handle, launch shapes and timed loop with qgpu_set_precision(QGPU_PRECISION_MIXED)"}
        eng.set_precision(PRECISION[args.precision])
    plain = None if args.no_plain else plain_form(systems, flush, args.plain_blocks, world, args.precision,
                                                  tune=not args.no_tune and not args.tuning)
    if rank != 0:
        return
    cpu = cpu_baseline(pool, args.cpu_steps) if pool else None
    if pool:
        pool.close()
    out = {
        "metric": METRIC, "value": round(ns_per_day, 3), "unit": "ns/day", "n_gpus": world, "steps": steps,
        "warmup": warm, "ms_per_step": round(ms / steps, 5), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPE[args.precision],
        "data": "synthetic (seeded water spheres, random-init)",
        "config": {"workload": WORKLOAD, "trajectories": ntraj, "atoms": natoms, "dt_fs": FS_PER_STEP, "nbcycle": NB,
                   "timed": f"{nblk} blocks of {NB} steps, each one CUDA-graph replay",
                   "l2": "flushed before every timed 10-step block (256 MB write on the engine stream)",
                   "parallelism": "replicas" if world > 1 else "single GPU, one handle",
                   "graph_branches": eng.branches(),
                   "precision": args.precision,
                   "launch_shapes": ({"lanes_water": tuning[0], "min_blocks_water": tuning[1],
                                      "lanes_solute": tuning[2], "lanes_qw": tuning[3], "unroll_water": tuning[4]}
                                     if tuning else "default")},
        "e2e": {"value": round(e2e, 3), "unit": "ns/day", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "how": "per 10-step block: qgpu_set_coords_all of x,v of all 32 trajectories from pinned memory, "
                       "qgpu_run_rows (the block's energy records of every trajectory into host arrays and a .en "
                       "frame per trajectory), qgpu_get_coords_all (host wall clock); qgpu_fep_start over the "
                       "21-window chain before, the .en files opened and closed inside the timed region",
                "en_bytes": int(en_bytes), "fep_frames_window0": fep_frames},
        "mixed_form": mixed,
        "roofline": roof,
        "kernel_share": share,
        "kernel_roofline": per_kernel,
        "kernel_us_per_step": us_per_step,
        "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")} if cpu else None,
        "plain_form": plain,
        "batched_over_plain": round(ns_per_day / plain["value"], 3) if plain else None,
        "clocks": clk,
        "gpu_launches": int(launches),
        "work": wc,
    }
    print(json.dumps(out))


def timed_blocks(eng, ext, flush, nblk: int, dist):
    """nblk 10-step graph replays on the engine's stream, each bracketed by
    CUDA events and preceded by an L2 flush (a 256 MB write); barrier and
    synchronize on both sides.  Returns (ms, the engine's kernel launches,
    the clocks sampled during the region); ms is the max over ranks."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nblk)]
    clocks = Clocks()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    l0 = eng.kernel_launches()
    with torch.cuda.stream(ext):
        for b in range(nblk):
            flush.fill_(float(b))
            ev[b][0].record(ext)
            eng.enqueue(NB, NB)
            ev[b][1].record(ext)
    eng.sync()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = eng.kernel_launches() - l0
    clk = clocks.stop()
    ms = sum(a.elapsed_time(b) for a, b in ev)
    if dist:
        ms = max_over_ranks(dist, ms, "cuda")
    return ms, launches, clk


def max_over_ranks(dist, value: float, device: str = "cpu") -> float:
    """The largest of every rank's timing (the job ends with its slowest rank)."""
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_ns_per_day(world: int, ntraj: int, steps: int, ms: float) -> float:
    """Whole-job ns/day: every rank advances ntraj trajectories by steps fs-steps
    in ms milliseconds (max over ranks)."""
    return world * ntraj * steps * FS_PER_STEP * 1e-6 * 86400.0 / (ms * 1e-3)


def ctypes_peak(eng, fn: str) -> float:
    """TFLOP/s of the library's in-run FMA-chain probe fn (qgpu_fp32_peak /
    qgpu_fp64_peak)."""
    import ctypes as C
    v = C.c_double()
    rc = getattr(eng.lib, fn)(C.byref(v))
    return v.value if rc == 0 else float("nan")


def committed_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary
    (profiles/traffic.json), or None when no capture was summarised."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            return json.load(f).get(kernel)
    except Exception:
        return None


if __name__ == "__main__":
    main()
