"""CPU oracle of the opening-criterion network (test infrastructure only).

FP64 restatement of the network the GPU evaluates and trains: 12 inputs,
two hidden layers of 64 SiLU units, one logit; weights and the activations
fed to each layer rounded to BF16 (round-to-nearest-even), straight-through
gradients; loss = weighted mean binary cross-entropy on the logit.
Parameter vector order: W1[64][12], b1[64], W2[64][64], b2[64], W3[64], b3.
"""
import numpy as np

H, I = 64, 12
NP = H * I + H + H * H + H + H + 1


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + H * I].reshape(H, I); o += H * I
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, W3, b3


def silu(z):
    return z / (1.0 + np.exp(-z))


def forward(p, x):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    X = bf16(x)
    Z1 = X @ bf16(W1).T + b1
    H1 = bf16(silu(Z1))
    Z2 = H1 @ bf16(W2).T + b2
    H2 = bf16(silu(Z2))
    z3 = H2 @ bf16(W3) + b3
    return z3, (X, Z1, H1, Z2, H2)


def loss_and_grad(p, x, y, w=None):
    """Summed weighted BCE and the gradient of the weighted mean."""
    y = np.asarray(y, dtype=np.float64)
    w = np.ones_like(y) if w is None else np.asarray(w, dtype=np.float64)
    W1, b1, W2, b2, W3, b3 = unpack(p)
    z3, (X, Z1, H1, Z2, H2) = forward(p, x)
    loss = np.sum(w * (np.maximum(z3, 0) - z3 * y + np.log1p(np.exp(-np.abs(z3)))))
    sig = lambda z: 1.0 / (1.0 + np.exp(-z))
    d = w * (sig(z3) - y) / w.sum()
    dsilu = lambda z: sig(z) * (1 + z * (1 - sig(z)))
    dZ2 = (d[:, None] * bf16(W3)[None, :]) * dsilu(Z2)
    dZ1 = (dZ2 @ bf16(W2)) * dsilu(Z1)
    g = np.concatenate([(dZ1.T @ X).ravel(), dZ1.sum(0), (dZ2.T @ H1).ravel(), dZ2.sum(0), d @ H2, [d.sum()]])
    return loss, g
