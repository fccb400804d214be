"""FP64 CPU oracle of the integration proposal network and its features.

Test infrastructure only: the parity tests and the gradient check import this
module to verify the CUDA kernels behind gg_mlp_features, gg_mlp_grad,
gg_mlp_adam and gg_mlp_infer.  The network has no counterpart in the
reference (GIMIC integrates planes on fixed grids, src/fgimic/integral.f90:
50-511); its behaviour is pinned by finite differences of this restatement
(tests/test_proposal.py) instead of by reference outputs.

Network: x (5) -> SiLU(W1 x + b1) (64) -> SiLU(W2 h1 + b2) (64) -> W3 h2 + b3.
Parameters are one flat vector laid out W1[64][5] b1[64] W2[64][64] b2[64]
W3[64] b3.  Loss: mean squared error over the batch.
"""
import numpy as np

N_IN, N_H = 5, 64
SIZES = [("W1", (N_H, N_IN)), ("b1", (N_H,)), ("W2", (N_H, N_H)), ("b2", (N_H,)), ("W3", (N_H,)), ("b3", (1,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    out, off = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = p[off:off + n].reshape(shape)
        off += n
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, x):
    w = unpack(np.asarray(p, dtype=np.float64))
    x = np.asarray(x, dtype=np.float64)
    z1 = x @ w["W1"].T + w["b1"]
    h1 = silu(z1)
    z2 = h1 @ w["W2"].T + w["b2"]
    h2 = silu(z2)
    return h2 @ w["W3"] + w["b3"][0], (z1, h1, z2, h2)


def loss_and_grad(p, x, t):
    """Mean squared error and its gradient with respect to the flat
    parameter vector, by backpropagation."""
    w = unpack(np.asarray(p, dtype=np.float64))
    x = np.asarray(x, dtype=np.float64)
    y, (z1, h1, z2, h2) = forward(p, x)
    n = len(t)
    err = y - np.asarray(t, dtype=np.float64)
    dy = 2.0 * err / n
    g = {"W3": h2.T @ dy, "b3": np.array([dy.sum()])}
    d2 = np.outer(dy, w["W3"]) * dsilu(z2)
    g["W2"] = d2.T @ h1
    g["b2"] = d2.sum(axis=0)
    d1 = (d2 @ w["W2"]) * dsilu(z1)
    g["W1"] = d1.T @ x
    g["b1"] = d1.sum(axis=0)
    flat = np.concatenate([g[name].reshape(-1) for name, _ in SIZES])
    return float(np.mean(err ** 2)), flat


def adam(p, grad, m, v, lr, beta1, beta2, eps, step):
    """One bias-corrected Adam step; returns new (p, m, v)."""
    m = beta1 * m + (1.0 - beta1) * grad
    v = beta2 * v + (1.0 - beta2) * grad * grad
    mh = m / (1.0 - beta1 ** step)
    vh = v / (1.0 - beta2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v


def bf16(a):
    """Round to the nearest bfloat16 (ties to even), returned as float32."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def infer_bf16(p, x):
    """Inference as the bf16 kernel does it: weights, inputs and hidden
    activations rounded to bf16, arithmetic in float64 here."""
    w = unpack(bf16(np.asarray(p, dtype=np.float32)).astype(np.float64))
    x = bf16(x).astype(np.float64)
    h1 = bf16(silu(x @ w["W1"].T + w["b1"])).astype(np.float64)
    h2 = bf16(silu(h1 @ w["W2"].T + w["b2"])).astype(np.float64)
    return h2 @ w["W3"] + w["b3"][0]


def features(atom_xyz, shell_atom, shell_min_exp, pts, uv):
    """The five inputs: u/8, v/8, ln of the distances to the nearest and
    second-nearest nucleus (floored at 0.05 Bohr), and
    log10(1e-6 + sum_s sqrt(a_s) exp(-a_s d_s^2)) / 3."""
    pts = np.asarray(pts, dtype=np.float64).reshape(-1, 3)
    uv = np.asarray(uv, dtype=np.float64).reshape(-1, 2)
    d2 = ((pts[:, None, :] - np.asarray(atom_xyz)[None, :, :]) ** 2).sum(axis=2)
    s = np.sort(d2, axis=1)
    n1 = s[:, 0]
    n2 = s[:, 1] if s.shape[1] > 1 else s[:, 0]
    a = np.asarray(shell_min_exp, dtype=np.float64)
    ds = d2[:, np.asarray(shell_atom)]
    dens = (np.sqrt(a)[None, :] * np.exp(-a[None, :] * ds)).sum(axis=1)
    return np.stack([uv[:, 0] * 0.125, uv[:, 1] * 0.125, np.log(np.maximum(np.sqrt(n1), 0.05)),
                     np.log(np.maximum(np.sqrt(n2), 0.05)), np.log10(1e-6 + dens) / 3.0], axis=1)
