"""The learned lambda schedule trained on window data the engine generates,
judged where window placement matters.

Two families of seeded 16 A droplets with 8 Q atoms, 21 uniform windows each
(lambda_A from 0 to 1), run as one batch per system: 1,000 equilibration
steps, a pilot of 1,000 steps and a long run of 8,000 steps with the device
FEP sums on (energies every 10 steps).
  * discharge (the config 3 windows): charges N(0, sigma) in state A, zero in
    state B, same LJ; s(lambda) is nearly flat;
  * vanish (towards a decoupling end point): the same discharge, and the Q
    atoms' LJ parameters (sqrt A, sqrt B) scaled by 0.12 in state B; waters
    come close to the weakly repulsive Q atoms near pure state B, so the
    energy-gap spread grows steeply there, the case that uniform windows
    sample badly.
The network (the library's GPU kernels) is trained on 6 systems of each
family -- pilot statistics in, long-run log-spread out -- and places 11
windows on 2 held-out systems of each family from their pilots alone.  Each
placement is scored by the expected squared error of the summed Zwanzig
estimates under the long-run spread curve (Gaussian gaps, tests/mlp_ref.py
schedule_mse); at a fixed window count that error is inversely proportional
to the sampling, so the ratio learned / uniform is the ratio of GPU time
needed to reach the same Delta-G error.

Asserted: training fits (loss down 5x); on the vanish family the learned
schedule needs at most 0.8 of the uniform schedule's GPU time (median); on
the discharge family it is no worse than uniform by more than 5 %."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KT = 0.001986 * 300.0
LAM = np.linspace(0.0, 1.0, 21)
NSYS, NTRAIN = 16, 12


def _windows(k):
    from qsource_gb300 import synth
    rng = np.random.default_rng(500 + k)
    qa = synth.neutral_charges(rng, 8, [0.3, 0.45, 0.6][k % 3])
    vanish = k % 2 == 1
    return [synth.synthetic(16.0, 8, 8, np.stack([qa, np.zeros(8)], 1), (l, 1.0 - l), 9000 + 37 * k,
                            qvdw=vanish, q_lj_scale=(0.12, 0.12)) for l in LAM]


def _stats(k):
    from qsource_gb300.engine import Engine
    e = Engine(_windows(k))
    chain = list(range(len(LAM)))
    e.run(1000)
    e.fep_start(chain, KT, 0)
    e.run(1000, ene_every=10, collect=False)
    pilot = e.fep_result()[3]
    e.fep_start(chain, KT, 0)
    e.run(8000, ene_every=10, collect=False)
    long_ = e.fep_result()[3]
    e.close()
    return pilot, long_


def test_learned_schedule_on_engine_windows(engine_lib):
    from mlp_ref import schedule_mse
    from qsource_gb300.schedule import MLP, features, learned_schedule, place, window_spread
    data = [_stats(k) for k in range(NSYS)]
    X = np.concatenate([features(LAM, p, KT) for p, _ in data[:NTRAIN]])
    Y = np.concatenate([np.log(window_spread(LAM, l)) for _, l in data[:NTRAIN]]).astype(np.float32)
    net = MLP(seed=2)
    loss = net.train_batches(X, Y, epochs=40, iters=25, lr=3e-3)
    print(f"engine schedule training loss {loss[0]:.4g} -> {loss[-1]:.4g}")
    assert loss[-1] < 0.2 * loss[0]
    rep = {"discharge": [], "vanish": []}
    for k in range(NTRAIN, NSYS):
        pilot, long_ = data[k]
        s_long = window_spread(LAM, long_)
        s = lambda x, s_long=s_long: np.interp(x, LAM, s_long)
        uni = schedule_mse(s, np.linspace(0, 1, 11), KT, 200)
        lrn = schedule_mse(s, learned_schedule(net, LAM, pilot, KT, 11)[0], KT, 200)
        raw = schedule_mse(s, place(LAM, window_spread(LAM, pilot), 11), KT, 200)
        opt = schedule_mse(s, place(LAM, s_long, 11), KT, 200)
        rep["vanish" if k % 2 else "discharge"].append(
            {"learned/uniform": lrn / uni, "raw_pilot/uniform": raw / uni, "best/uniform": opt / uni,
             "spread_end/spread_mid": float(s_long[0] / s_long[10])})
    med = {fam: {key: float(np.median([r[key] for r in rows])) for key in rows[0]} for fam, rows in rep.items()}
    print("engine schedule report", json.dumps(med))
    assert med["vanish"]["spread_end/spread_mid"] > 2.0      # the curved case is curved
    assert med["vanish"]["learned/uniform"] <= 0.8
    assert med["discharge"]["learned/uniform"] <= 1.05
