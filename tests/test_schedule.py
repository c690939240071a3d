"""Host-side parts of the learned lambda schedule (no GPU): window placement
by thermodynamic length, the network's input rows, and the CPU reference of
the network (its gradient against finite differences)."""
import numpy as np

from mlp_ref import loss_and_grad, s_curve, schedule_mse


def test_place_equalises_thermodynamic_length():
    from qsource_gb300.schedule import place
    lam = np.linspace(0, 1, 11)
    assert np.allclose(place(lam, np.ones(11), 6), np.linspace(0, 1, 6))
    s = 1.0 + 20.0 * lam ** 3
    w = place(lam, s, 9)
    assert w[0] == 0.0 and w[-1] == 1.0 and np.all(np.diff(w) > 0)
    # equal increments of the integral of the piecewise-linear s
    fine = np.linspace(0, 1, 20001)
    sf = np.interp(fine, lam, s)
    L = np.concatenate([[0], np.cumsum(0.5 * (sf[1:] + sf[:-1]) * np.diff(fine))])
    inc = np.diff(np.interp(w, fine, L))
    assert np.allclose(inc, inc.mean(), rtol=2e-3)
    # windows crowd where s is large
    assert np.diff(w)[-1] < np.diff(w)[0]


def test_thermodynamic_length_beats_uniform_with_true_spread():
    from qsource_gb300.schedule import place
    rng = np.random.default_rng(3)
    kT = 0.596
    for _ in range(5):
        s = s_curve(rng)
        lam = np.linspace(0, 1, 41)
        w = place(lam, np.array([s(x) for x in lam]), 21)
        assert schedule_mse(s, w, kT, 200) < schedule_mse(s, np.linspace(0, 1, 21), kT, 200)


def test_features_rows():
    from qsource_gb300.schedule import NF, features
    lam = np.linspace(1, 0, 5)
    st = np.zeros((5, 7))
    st[:, 0] = 10
    st[:, 2] = 0.04
    st[:, 5] = 0.04
    X = features(lam, st, 0.6)
    assert X.shape == (5, NF) and X.dtype == np.float32 and np.all(np.isfinite(X))
    assert X[0, 9] == 0.0 and X[-1, 8] == 0.0      # no backward / forward neighbour at the ends


def test_reference_gradient_matches_finite_differences():
    """The backward formulas of the reference (without BF16 rounding) against
    central differences of its loss, for weights of every layer and biases."""
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.1, 128 * 16 + 128 + 128 * 128 + 128 + 16 * 128 + 16)
    X = rng.normal(0, 1, (20, 16))
    Y = rng.normal(0, 1, 20)
    _, g = loss_and_grad(p, X, Y, exact=True)
    for idx in (3, 128 * 16 + 5, 128 * 16 + 128 + 1000, 128 * 16 + 128 + 128 * 128 + 7,
                128 * 16 + 128 + 128 * 128 + 128 + 50, len(p) - 16):
        h = 1e-5
        pp, pm = p.copy(), p.copy()
        pp[idx] += h
        pm[idx] -= h
        fd = (loss_and_grad(pp, X, Y, True)[0] - loss_and_grad(pm, X, Y, True)[0]) / (2 * h)
        assert abs(fd - g[idx]) <= 1e-5 * max(abs(fd), 1e-2), (idx, fd, g[idx])
