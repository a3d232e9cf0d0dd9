"""CPU FP64 restatement of the chemistry-surrogate network (TEST INFRASTRUCTURE ONLY).

The network of gdtk_gb300/csrc/surrogate.cpp: layers l = 0..depth, h_{l+1} = GELU(h_l W_l^T + b_l)
for the hidden layers (tanh-form GELU), a linear output layer, and the loss
    L = (1/B) sum_rows sum_n w_n (out_n - y_n)^2
on standardised inputs and targets.  The surrogate has no counterpart in the reference, so this
module is the oracle of the library's forward and backward kernels (mlp_kernels.cu): the
gradient of L with respect to every weight and bias, in FP64 by reverse-mode differentiation
written out by hand (checked here against central finite differences).

With bf16=True the values the GPU kernels hold in BF16 are rounded to BF16 at the same points
(weights, inputs, hidden activations, and the output / pre-activation gradients that feed the
weight-gradient and input-gradient products); everything else stays FP64.  What then remains
between the two is FP32 accumulation order.
"""
import numpy as np

C_GELU = 0.7978845608028654   # sqrt(2 / pi)


def bf16(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(C_GELU * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    t = np.tanh(C_GELU * (x + 0.044715 * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * C_GELU * (1.0 + 3.0 * 0.044715 * x * x)


def forward(layers, X, bf=False):
    """layers: [(W (out, in), b (out,))]; X (B, in) standardised.  Returns (out, cache)."""
    r = bf16 if bf else (lambda v: np.asarray(v, np.float64))
    h = r(X)
    cache = []
    for l, (W, b) in enumerate(layers):
        z = h @ r(W).T + b
        if l < len(layers) - 1:
            cache.append((h, z))
            h = r(gelu(z))
        else:
            cache.append((h, None))
            out = z
    return out, cache


def loss_and_grads(layers, X, Y, w, bf=False, quantile=None):
    """(L, [(dW_l, db_l)]) for standardised X (B, in), Y (B, out), output weights w (out,): the
    weighted squared error, or with `quantile` the pinball loss of output column 0
    (mean of max(q r, (q - 1) r), r = Y - out)."""
    r = bf16 if bf else (lambda v: np.asarray(v, np.float64))
    B = X.shape[0]
    out, cache = forward(layers, X, bf)
    if quantile is None:
        d = out - Y
        L = float(np.sum(w[None, :] * d * d)) / B
        g = 2.0 * w[None, :] * d / B          # dL/d(out), the fp32 copy
    else:
        res = Y[:, 0] - out[:, 0]
        L = float(np.sum(np.where(res > 0, quantile * res, (quantile - 1.0) * res))) / B
        g = np.zeros_like(out)
        g[:, 0] = np.where(res > 0, -quantile, 1.0 - quantile) / B
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        h, _ = cache[l]
        g16 = r(g)
        dW = g16.T @ h
        db = g.sum(axis=0)
        grads[l] = (dW, db)
        if l > 0:
            W = r(layers[l][0])
            z_prev = cache[l - 1][1]
            g = (g16 @ W) * gelu_grad(z_prev)
    return L, grads


def finite_difference_check(layers, X, Y, w, n_probe=20, eps=1e-6, seed=0, quantile=None):
    """Largest relative difference between the analytic FP64 gradient and central differences
    at n_probe random parameters."""
    rng = np.random.Generator(np.random.PCG64(seed))
    _, grads = loss_and_grads(layers, X, Y, w, quantile=quantile)
    worst = 0.0
    for _ in range(n_probe):
        l = int(rng.integers(len(layers)))
        which = int(rng.integers(2))
        P = layers[l][which]
        idx = tuple(int(rng.integers(s)) for s in P.shape)
        old = P[idx]
        P[idx] = old + eps
        Lp, _ = loss_and_grads(layers, X, Y, w, quantile=quantile)
        P[idx] = old - eps
        Lm, _ = loss_and_grads(layers, X, Y, w, quantile=quantile)
        P[idx] = old
        fd = (Lp - Lm) / (2 * eps)
        an = grads[l][which][idx]
        worst = max(worst, abs(fd - an) / max(abs(fd), abs(an), 1e-8))
    return worst
