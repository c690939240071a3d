"""Learned lambda-window schedule.

The reference runs FEP lambda windows one after another on a schedule the
user writes down (typically uniform steps, e.g. tests/exclude_tests/inputs/
excl/gen_inps.pl steps lambda by 0.02).  This module places windows from a
short pilot run instead:

1. A pilot batch of uniform windows runs for a short time with the device's
   streaming FEP sums on (qgpu_fep_start).  Each window w gives the mean,
   variance and skew of the forward and backward energy gaps dV
   (qgpu_fep_result).
2. Per pilot window the MLP (qgpu_mlp_*: BF16 tensor-core products, FP32
   accumulation, trained on the GPU by the library's own kernels) maps those
   short-run statistics to s(lambda) = the standard deviation of
   dV/dlambda = V_B - V_A that a long run would give.  Short runs estimate it
   poorly where the gap distribution is wide and slowly sampled -- exactly
   where windows are needed.
3. Windows are placed at equal increments of the thermodynamic length
   L(lambda) = integral of s, so that every interval carries the same gap
   spread s * dlambda (the spacing that minimises the summed FEP variance for
   a fixed window count).  The uniform schedule is the fallback whenever the
   network is missing or its prediction is not finite and positive.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi

NF = 16          # padded input width of the network
BATCH = 64       # rows per call


def features(lam: np.ndarray, stats: np.ndarray, kT: float) -> np.ndarray:
    """Input rows of the network, one per pilot window.

    lam[n]: lambda of state A of each window (state B has 1 - lambda);
    stats[n, 7]: qgpu_fep_result's per-window frames, mean / variance / skew
    of dV forward and of dV backward.  Gaps are divided by the lambda step to
    neighbouring windows (dV ~ (V_B - V_A) dlambda) and by kT.
    """
    n = len(lam)
    X = np.zeros((n, NF), dtype=np.float32)
    dl = np.abs(np.gradient(lam)) if n > 1 else np.ones(1)
    for w in range(n):
        f_mu, f_var, f_sk = stats[w, 1:4]
        b_mu, b_var, b_sk = stats[w, 4:7]
        has_f, has_b = w + 1 < n, w > 0
        sf = np.sqrt(max(f_var, 0.0)) / (dl[w] * kT) if has_f else 0.0
        sb = np.sqrt(max(b_var, 0.0)) / (dl[w] * kT) if has_b else 0.0
        s_pool = np.mean([v for v, h in ((sf, has_f), (sb, has_b)) if h]) if (has_f or has_b) else 0.0
        X[w, :10] = [lam[w], np.log1p(s_pool), np.log1p(sf), np.log1p(sb), f_sk if has_f else 0.0,
                     b_sk if has_b else 0.0, (f_mu / (dl[w] * kT)) / 100.0 if has_f else 0.0,
                     (b_mu / (dl[w] * kT)) / 100.0 if has_b else 0.0, float(has_f), float(has_b)]
        X[w, 10] = np.log(max(stats[w, 0], 1.0)) / 10.0
    return X


def window_spread(lam: np.ndarray, stats: np.ndarray) -> np.ndarray:
    """s(lambda) at each window from qgpu_fep_result statistics: the pooled
    standard deviation of the forward and backward energy gaps divided by the
    lambda step (kcal/mol per unit lambda) -- the network's training target
    when stats come from a long run."""
    n = len(lam)
    dl = np.abs(np.gradient(lam)) if n > 1 else np.ones(1)
    out = np.empty(n)
    for w in range(n):
        v = ([stats[w, 2]] if w + 1 < n else []) + ([stats[w, 5]] if w > 0 else [])
        out[w] = np.sqrt(max(float(np.mean(v)), 0.0)) / dl[w]
    return out


def place(lam_pilot: np.ndarray, s_pilot: np.ndarray, nwin: int) -> np.ndarray:
    """nwin windows from 0 to 1 at equal increments of the thermodynamic
    length of the piecewise-linear s(lambda) through the pilot points."""
    order = np.argsort(lam_pilot)
    x = np.asarray(lam_pilot, dtype=np.float64)[order]
    s = np.maximum(np.asarray(s_pilot, dtype=np.float64)[order], 1e-9)
    seg = 0.5 * (s[1:] + s[:-1]) * np.diff(x)
    L = np.concatenate([[0.0], np.cumsum(seg)])
    targets = np.linspace(0.0, L[-1], nwin)
    out = np.empty(nwin)
    for k, t in enumerate(targets):
        j = min(np.searchsorted(L, t, side="right") - 1, len(seg) - 1)
        j = max(j, 0)
        # inside segment j, s varies linearly: solve the quadratic for the offset
        a, b, h = s[j], s[j + 1], x[j + 1] - x[j]
        r = t - L[j]
        if abs(b - a) < 1e-12 * max(a, b):
            u = r / a
        else:
            k2 = (b - a) / h
            u = (-a + np.sqrt(max(a * a + 2.0 * k2 * r, 0.0))) / k2
        out[k] = np.clip(x[j] + u, 0.0, 1.0)
    out[0], out[-1] = x[0], x[-1]
    return out


class MLP:
    """The schedule network: FP32 parameters on the host, training and
    inference through the library's kernels."""

    def __init__(self, seed: int = 0, lib=None):
        self.lib = lib or abi.load_library()
        self.n = int(self.lib.qgpu_mlp_nparams())
        rng = np.random.default_rng(seed)
        p = np.zeros(self.n, dtype=np.float32)
        H, F, O = 128, NF, 16
        o = 0
        for rows, cols in ((H, F), (H, None), (H, H), (H, None), (O, H), (O, None)):
            if cols is None:
                o += rows
                continue
            p[o:o + rows * cols] = rng.normal(0.0, np.sqrt(1.0 / cols), rows * cols)
            o += rows * cols
        self.params = p
        self.m = np.zeros(self.n, dtype=np.float32)
        self.v = np.zeros(self.n, dtype=np.float32)
        self.steps = 0

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(abi.last_error(self.lib))

    def predict(self, X: np.ndarray) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        out = np.zeros(len(X), dtype=np.float32)
        for a in range(0, len(X), BATCH):
            xb = np.ascontiguousarray(X[a:a + BATCH])
            ob = np.zeros(len(xb), dtype=np.float32)
            self._check(self.lib.qgpu_mlp_predict(abi.ptr(self.params), abi.ptr(xb), len(xb), abi.ptr(ob)))
            out[a:a + BATCH] = ob
        return out

    def train_batches(self, X: np.ndarray, Y: np.ndarray, epochs: int, iters: int = 20, lr: float = 1e-3, seed: int = 0):
        """Adam over more than 64 rows: each epoch walks a seeded shuffle of
        the rows in batches of up to 64, `iters` steps per batch (the Adam
        state carries over).  Returns the loss of the last step of each batch."""
        X = np.asarray(X, dtype=np.float32)
        Y = np.asarray(Y, dtype=np.float32)
        rng = np.random.default_rng(seed)
        out = []
        for _ in range(epochs):
            idx = rng.permutation(len(X))
            for a in range(0, len(X), BATCH):
                sel = idx[a:a + BATCH]
                loss, _ = self.train(X[sel], Y[sel], iters, lr)
                out.append(float(loss[-1]))
        return np.array(out)

    def train(self, X: np.ndarray, Y: np.ndarray, iters: int, lr: float = 1e-3):
        """Full-batch Adam on up to 64 rows; returns (loss per step, last gradient)."""
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        if len(X) > BATCH:
            raise ValueError("at most 64 training rows per call")
        loss = np.zeros(iters, dtype=np.float32)
        grad = np.zeros(self.n, dtype=np.float32)
        self._check(self.lib.qgpu_mlp_train(abi.ptr(self.params), abi.ptr(self.m), abi.ptr(self.v), abi.ptr(X),
                                            abi.ptr(Y), len(X), iters, C.c_float(lr), self.steps, abi.ptr(loss),
                                            abi.ptr(grad)))
        self.steps += iters
        return loss, grad


def learned_schedule(net: MLP | None, lam_pilot: np.ndarray, stats: np.ndarray, kT: float, nwin: int):
    """Window lambdas from a pilot run: the network's s(lambda) (exp of its
    output) at the pilot windows, then equal thermodynamic-length spacing.
    Falls back to uniform spacing without a usable prediction."""
    uniform = np.linspace(0.0, 1.0, nwin)
    if net is None:
        return uniform, None
    s = np.exp(net.predict(features(lam_pilot, stats, kT)).astype(np.float64))
    if not np.all(np.isfinite(s)) or np.any(s <= 0):
        return uniform, None
    return place(lam_pilot, s, nwin), s
