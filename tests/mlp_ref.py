"""CPU reference of the schedule network (test infrastructure): the same
3-layer tanh MLP as the library's kernels, with the kernels' BF16 rounding of
every tensor-core operand (inputs, weights, activations, backward gradients)
and FP64 sums.  Also a Gaussian model of FEP windows used to score schedules."""
import numpy as np

F, H, O = 16, 128, 16


def bf16(a):
    """Round float32 values to bfloat16 (nearest, ties to even), as float64."""
    a = np.asarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p)
    o = 0
    out = []
    for n in (H * F, H, H * H, H, O * H, O):
        out.append(p[o:o + n].astype(np.float64))
        o += n
    W1, b1, W2, b2, W3, b3 = out
    return W1.reshape(H, F), b1, W2.reshape(H, H), b2, W3.reshape(O, H), b3


def _r(exact):
    return (lambda a: np.asarray(a, dtype=np.float64)) if exact else bf16


def forward(p, X, exact=False):
    """exact=True: no BF16 rounding (the mathematical network)."""
    bf16 = _r(exact)
    W1, b1, W2, b2, W3, b3 = unpack(p)
    x = bf16(X)
    t = (lambda a: np.tanh(a)) if exact else (lambda a: np.tanh(a.astype(np.float32)).astype(np.float64))
    h1 = t(x @ bf16(W1).T + b1)
    h2 = t(bf16(h1) @ bf16(W2).T + b2)
    y = bf16(h2) @ bf16(W3).T + b3
    return x, h1, h2, y


def loss_and_grad(p, X, Y, exact=False):
    bf16 = _r(exact)
    W1, b1, W2, b2, W3, b3 = unpack(p)
    n = len(X)
    x, h1, h2, y = forward(p, X, exact)
    e = y[:, 0] - Y
    loss = float(np.mean(e * e))
    gy = np.zeros_like(y)
    gy[:, 0] = 2.0 * e / n
    g3 = bf16(gy)
    gW3 = g3.T @ bf16(h2)
    gb3 = gy.sum(0)
    g2f = (g3 @ bf16(W3)) * (1.0 - h2 * h2)
    g2 = bf16(g2f)
    gW2 = g2.T @ bf16(h1)
    gb2 = g2f.sum(0)
    g1f = (g2 @ bf16(W2)) * (1.0 - h1 * h1)
    g1 = bf16(g1f)
    gW1 = g1.T @ x
    gb1 = g1f.sum(0)
    grad = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, grad


# ---------------------------------------------------------------- FEP model
def s_curve(rng):
    """A random smooth, positive spread s(lambda) of V_B - V_A (kcal/mol),
    steep towards one end as a charging free energy is."""
    a = rng.uniform(0.5, 2.0)
    b = rng.uniform(3.0, 25.0)
    p = rng.uniform(2.0, 5.0)
    flip = rng.random() < 0.5
    return lambda lam: a + b * ((1.0 - lam) if flip else lam) ** p


def pilot_stats(rng, s, lam, kT, nsamp):
    """Per pilot window the 7 statistics qgpu_fep_result reports, from nsamp
    short-run samples of dV = dlambda (V_B - V_A).  A short run sees a
    narrowed gap distribution where the true one is wide (slow modes not
    sampled): the sampled spread is s / (1 + s / 12)."""
    n = len(lam)
    st = np.zeros((n, 7))
    for w in range(n):
        sw = s(lam[w])
        seen = sw / (1.0 + sw / 12.0)
        for d, nb in ((0, w + 1), (1, w - 1)):
            if 0 <= nb < n:
                dl = lam[nb] - lam[w]
                dv = dl * rng.normal(0.0, seen, nsamp)
                st[w, 1 + 3 * d] = dv.mean()
                st[w, 2 + 3 * d] = dv.var()
                st[w, 3 + 3 * d] = 0.0
        st[w, 0] = nsamp
    return st


def schedule_mse(s, lams, kT, nsamp):
    """Expected squared error of the summed Zwanzig estimates of a window
    schedule with Gaussian gaps (delta method): sum over intervals of
    kT^2 (exp(sigma^2) - 1)/nsamp, sigma = s(mid) dlambda / kT."""
    lams = np.sort(np.asarray(lams))
    mid = 0.5 * (lams[1:] + lams[:-1])
    sig = np.array([s(m) for m in mid]) * np.diff(lams) / kT
    return float(np.sum(kT * kT * np.expm1(np.minimum(sig * sig, 700.0)) / nsamp))
