"""Precision form on one system (the 30 A sphere with the 2,000-atom chain
and 50 Q atoms, 2 states): 10,000 MD steps of the persistent mixed-precision
engine; every 500 steps the coordinates are taken and the forces and
per-state energies are evaluated on the same coordinates by

  * the engine's step precision (FP32 pair and bonded terms, FP32 energy sums:
    what every unrecorded step uses),
  * the engine's drop-in FP64-energy evaluation (what recorded steps and
    qgpu_forces use),
  * the FP64 oracle.

Reported (printed) and asserted at every sample: force relative RMS
sqrt(sum|dF|^2 / sum|F|^2) <= 1e-5; per-state Q energies within 1e-6 relative
(2e-3 kcal/mol absolute for terms below 2,000 kcal/mol) for the FP64 form and
within 1e-5 relative (2e-2 kcal/mol absolute below 2,000) for the step form.
The file name makes pytest run it late (it takes about a minute)."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

Q_KEYS = ["qq_el", "qq_vdw", "qp_el", "qp_vdw", "qw_el", "qw_vdw", "q_bond", "q_angle", "q_torsion", "q_improper"]


def _rel(a, b):
    return float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b ** 2)))


def _qerr(EQ, EQo):
    worst = 0.0
    for q, qo in zip(EQ, EQo):
        for k in Q_KEYS:
            worst = max(worst, abs(q[k] - qo[k]) / max(abs(qo[k]), 2e-3 / 1e-6))
    return worst


def test_precision_form_over_10000_steps(engine_lib):
    from oracle.oracle import Oracle
    from qsource_gb300 import synth
    from qsource_gb300.abi import QGPU_TERMS_STEP_PRECISION
    from qsource_gb300.engine import Engine
    s = synth.config(2)
    e = Engine(s)
    probe = Engine(s)
    o = Oracle(s)
    rows = []
    for blk in range(20):
        e.run(500)
        x, v = e.coords(0)
        probe.set_coords(0, x, v)
        probe.make_pair_lists()
        d32, _, EQ32 = probe.pot_energy(0, terms=0x1F | QGPU_TERMS_STEP_PRECISION)
        d64, _, EQ64 = probe.pot_energy(0, terms=0x1F)
        o.set_coords(x, v)
        o.make_pair_lists()
        do, _, EQo = o.pot_energy(0x1F)
        rows.append({"step": 500 * (blk + 1), "force_relrms_step": _rel(d32, do), "force_relrms_fp64": _rel(d64, do),
                     "q_energy_rel_step": _qerr(EQ32, EQo), "q_energy_rel_fp64": _qerr(EQ64, EQo)})
    print("precision report", json.dumps({
        "force_relrms_step_max": max(r["force_relrms_step"] for r in rows),
        "force_relrms_fp64_max": max(r["force_relrms_fp64"] for r in rows),
        "q_energy_rel_step_max": max(r["q_energy_rel_step"] for r in rows),
        "q_energy_rel_fp64_max": max(r["q_energy_rel_fp64"] for r in rows),
        "samples": len(rows)}))
    for r in rows:
        assert r["force_relrms_step"] <= 1e-5 and r["force_relrms_fp64"] <= 1e-5, r
        assert r["q_energy_rel_fp64"] <= 1e-6, r
        assert r["q_energy_rel_step"] <= 1e-5, r
