"""CPU restatement of the warm-start network (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline may import
this module, and only as the checker of the GPU kernels in
experience-of-using-gpu-in-power-flow-computation_gb300/csrc/mlp.cu.

The reference has no learned warm start (its Newton loop always starts from
v_inicial / theta_inicial, GPU/sistInfo.h:62-242), so there is nothing in the
reference to pin this oracle to: parity for the network is unpinned against
the reference.  The oracle is pinned instead by
  * a float64 finite-difference check of its own analytic gradients
    (``fd_check``), and
  * the algorithm being the textbook one: y = W2 gelu(W1 x + b1) + b2 ...,
    GELU(z) = z * Phi(z) with Phi the standard normal CDF, mean-squared error,
    Adam (Kingma & Ba 2015, Algorithm 1) with bias-corrected moments.

``emulate=True`` rounds at exactly the points where the GPU stores bf16:
normalised features, weights, hidden activations, dLoss/dy and the
pre-activation gradients; everything else is float64, so the GPU (fp32
accumulation) and this oracle differ only by accumulation rounding and by the
rare bf16 value that lands on the other side of a rounding boundary.
"""
import numpy as np
from scipy.special import erf

SQRT1_2 = 0.7071067811865476
INV_SQRT_2PI = 0.3989422804014327


def bf16(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z * SQRT1_2))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z * SQRT1_2)) + z * INV_SQRT_2PI * np.exp(-0.5 * z * z)


def _r(x, emulate):
    return bf16(x) if emulate else np.asarray(x, np.float64)


def _split(params):
    """[(W, b)...] with an optional linear skip last as (S, None)."""
    if params and params[-1][1] is None:
        return params[:-1], params[-1][0]
    return params, None


def forward(params, Xn, emulate=True):
    """params = [(W [out, in], b [out]), ...] (+ (S [out, in], None): a linear
    skip y += S x summed with the output layer); returns (y, cache)."""
    params, S = _split(params)
    h = _r(Xn, emulate)
    cache = [h]
    zs = []
    n_l = len(params)
    for l, (W, b) in enumerate(params):
        z = h @ _r(W, emulate).T + np.asarray(b, np.float64)
        if l == n_l - 1:
            if S is not None:
                z = z + cache[0] @ _r(S, emulate).T
            return z, (cache, zs)
        zs.append(z)
        h = _r(gelu(z), emulate)
        cache.append(h)


def loss_and_grads(params, Xn, Yn, emulate=True, metric=None):
    """Loss over all rows and its gradients [(dW, db), ...] as the GPU's
    backward pass forms them.  metric None: mean squared error; metric =
    (A, lam): (sum_rows |e A|^2 + lam |e|^2) / (rows * n_out), with r = e A
    formed from bf16 e and bf16 A and r A^T from bf16 r, as on the GPU."""
    y, (hs, zs) = forward(params, Xn, emulate)
    params, S = _split(params)
    n, n_out = y.shape
    d = y - np.asarray(Yn, np.float64)
    if metric is None:
        loss = float(np.sum(d * d) / (n * n_out))
        g = _r(d * (2.0 / (n * n_out)), emulate)
    else:
        A, lam = metric
        Ar = _r(np.asarray(A, np.float64), emulate)
        r = _r(d, emulate) @ Ar
        q = _r(r, emulate) @ Ar.T
        loss = float((np.sum(r * r) + lam * np.sum(d * d)) / (n * n_out))
        g = _r((q + lam * d) * (2.0 / (n * n_out)), emulate)
    skip = [(g.T @ hs[0], None)] if S is not None else []
    grads = [None] * len(params)
    for l in range(len(params) - 1, -1, -1):
        W = _r(params[l][0], emulate)
        grads[l] = (g.T @ hs[l], g.sum(axis=0))
        if l > 0:
            g = _r((g @ W) * gelu_grad(zs[l - 1]), emulate)
    return loss, grads + skip


def adam_step(params, grads, state, t, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (t = 1 for the first step); state = [(mW, vW, mb, vb)]."""
    out, new_state = [], []
    for (W, b), (gW, gb), (mW, vW, mb, vb) in zip(params, grads, state):
        res = []
        for p, g, m, v in ((W, gW, mW, vW), (b, gb, mb, vb)):
            if p is None:
                res.append((None, None, None))
                continue
            m = b1 * m + (1 - b1) * g
            v = b2 * v + (1 - b2) * g * g
            p = p - lr * (m / (1 - b1 ** t)) / (np.sqrt(v / (1 - b2 ** t)) + eps)
            res.append((p, m, v))
        out.append((res[0][0], res[1][0]))
        new_state.append((res[0][1], res[0][2], res[1][1], res[1][2]))
    return out, new_state


def fd_check(params, Xn, Yn, n_probe=20, h=1e-5, seed=0):
    """Largest relative difference between analytic (float64, no rounding)
    and central finite-difference gradients at n_probe random parameters."""
    rng = np.random.default_rng(seed)
    params = [(np.array(W, np.float64), None if b is None else np.array(b, np.float64)) for W, b in params]
    _, grads = loss_and_grads(params, Xn, Yn, emulate=False)
    worst = 0.0
    for _ in range(n_probe):
        l = int(rng.integers(len(params)))
        which = int(rng.integers(2)) if params[l][1] is not None else 0
        arr = params[l][which]
        idx = tuple(int(rng.integers(s)) for s in arr.shape)
        old = arr[idx]
        arr[idx] = old + h
        lp, _ = loss_and_grads(params, Xn, Yn, emulate=False)
        arr[idx] = old - h
        lm, _ = loss_and_grads(params, Xn, Yn, emulate=False)
        arr[idx] = old
        fd = (lp - lm) / (2 * h)
        an = grads[l][which][idx]
        worst = max(worst, abs(fd - an) / max(1e-8, abs(fd) + abs(an)))
    return worst
