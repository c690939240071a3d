"""The learned lambda schedule trained on window data the engine generates.

Sixteen seeded 16 A droplets with 8 Q atoms (charges N(0, sigma), sigma 0.3 /
0.45 / 0.6, neutralised, discharged from state A to B; every other system also
changes the Q atoms' LJ type, hard to soft), 11 uniform windows each, batched
per system: 1,000 equilibration steps, a pilot of 1,000 steps and a long run of
8,000 steps with the device FEP sums on (energies every 10 steps).  The network
(the library's GPU kernels) is trained on 12 systems -- pilot statistics in,
long-run log-spread out -- and places 11 windows on the 4 held-out systems from
their pilots alone.  Scored with the long-run spread curve (Gaussian-gap error
of the summed Zwanzig estimates, tests/mlp_ref.py schedule_mse) against uniform
windows and against placing by the pilot's raw spread.

Asserted: training fits (loss down 10x) and the held-out median error of the
learned schedule is no worse than uniform windows by more than 5 %.  On this
family s(lambda) is nearly flat, so the best possible placement gains only a
few per cent over uniform; the printed report gives the measured ratios."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KT = 0.001986 * 300.0
LAM = np.linspace(0.0, 1.0, 11)


def _windows(k):
    from qsource_gb300 import synth
    rng = np.random.default_rng(500 + k)
    qa = synth.neutral_charges(rng, 8, [0.3, 0.45, 0.6][k % 3])
    return [synth.synthetic(16.0, 8, 8, np.stack([qa, np.zeros(8)], 1), (1.0 - l, l), 9000 + 37 * k,
                            qvdw=(k % 2 == 1)) for l in LAM]


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
    return pilot, e.fep_result()[3]


def test_learned_schedule_on_engine_windows(engine_lib):
    from mlp_ref import schedule_mse
    from qsource_gb300.schedule import MLP, features, learned_schedule, place, window_spread
    data = [_stats(k) for k in range(16)]
    X = np.concatenate([features(LAM, p, KT) for p, _ in data[:12]])
    Y = np.concatenate([np.log(window_spread(LAM, l)) for _, l in data[:12]]).astype(np.float32)
    net = MLP(seed=2)
    loss = net.train_batches(X, Y, epochs=40, iters=25, lr=3e-3)
    assert loss[-1] < 0.1 * loss[0]
    rep = []
    for pilot, long_ in data[12:]:
        s_long = window_spread(LAM, long_)
        s = lambda x, s_long=s_long: np.interp(x, LAM, s_long)
        uni = schedule_mse(s, np.linspace(0, 1, 11), KT, 200)
        lrn = schedule_mse(s, learned_schedule(net, LAM, pilot, KT, 11)[0], KT, 200)
        raw = schedule_mse(s, place(LAM, window_spread(LAM, pilot), 11), KT, 200)
        opt = schedule_mse(s, place(LAM, s_long, 11), KT, 200)
        rep.append({"learned/uniform": lrn / uni, "raw_pilot/uniform": raw / uni, "best/uniform": opt / uni})
    med = {k: float(np.median([r[k] for r in rep])) for k in rep[0]}
    print("engine schedule report", json.dumps(med))
    assert med["learned/uniform"] <= 1.05
