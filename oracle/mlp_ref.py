"""CPU restatement of the learned-sampler network (test infrastructure only:
the checker for the device kernels, never on the product path).

Layers 2 -> 128 -> 128 -> 128 -> 1 with exact GELU, loss mean((y - t)^2).
`emulate=True` rounds exactly where the device does: the inputs of the two
tensor-core products (activations h1, h2 in the forward pass, dz3, dz2 in the
backward pass) and the weights W2, W3 to BFloat16 (round to nearest even),
everything else in Float64.  `emulate=False` is plain Float64, for finite
differences.  Parameter layout: W1[128][2], b1[128], W2[128][128], b2[128],
W3[128][128], b3[128], w4[128], b4 (33537 floats).
"""
from __future__ import annotations

import numpy as np
from scipy.special import expit

H = 128
oW1, ob1 = 0, 2 * H
oW2 = ob1 + H
ob2 = oW2 + H * H
oW3 = ob2 + H
ob3 = oW3 + H * H
ow4 = ob3 + H
ob4 = ow4 + H
NPARAM = ob4 + 1


def bf16(a):
    """Round to the nearest BFloat16 (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


GELU_K = 2.0 * np.sqrt(2.0 / np.pi)
GELU_A = 0.044715


def gelu(z):
    # the tanh form of GELU (Hendrycks and Gimpel 2016): 0.5 z (1 + tanh(u)),
    # u = sqrt(2/pi) (z + 0.044715 z^3), written z sigmoid(2u)
    return z * expit(GELU_K * (z + GELU_A * z ** 3))


def dgelu(z):
    s = expit(GELU_K * (z + GELU_A * z ** 3))
    return s + z * s * (1.0 - s) * GELU_K * (1.0 + 3.0 * GELU_A * z * z)


def unpack(P):
    P = np.asarray(P, dtype=np.float64)
    return (P[oW1:ob1].reshape(H, 2), P[ob1:oW2], P[oW2:ob2].reshape(H, H), P[ob2:oW3],
            P[oW3:ob3].reshape(H, H), P[ob3:ow4], P[ow4:ob4], P[ob4])


def forward(P, x, emulate=True):
    W1, b1, W2, b2, W3, b3, w4, b4 = unpack(P)
    r = bf16 if emulate else (lambda a: np.asarray(a, dtype=np.float64))
    x = np.asarray(x, dtype=np.float64)
    z1 = x @ W1.T + b1
    h1 = r(gelu(z1))
    z2 = h1 @ r(W2).T + b2
    h2 = r(gelu(z2))
    z3 = h2 @ r(W3).T + b3
    h3 = gelu(z3)
    y = h3 @ w4 + b4
    return y, dict(x=x, z1=z1, h1=h1, z2=z2, h2=h2, z3=z3, h3=h3)


def gradient(P, x, t, emulate=True):
    """(grad, loss) of mean((net(x) - t)^2)."""
    W1, b1, W2, b2, W3, b3, w4, b4 = unpack(P)
    r = bf16 if emulate else (lambda a: np.asarray(a, dtype=np.float64))
    y, c = forward(P, x, emulate)
    n = len(y)
    e = y - np.asarray(t, dtype=np.float64)
    dy = 2.0 * e / n
    g = np.zeros(NPARAM)
    g[ob4] = dy.sum()
    g[ow4:ob4] = dy @ c["h3"]
    g3 = dy[:, None] * w4[None, :] * dgelu(c["z3"])
    g[ob3:ow4] = g3.sum(0)
    d3 = r(g3)
    g[oW3:ob3] = (d3.T @ c["h2"]).ravel()
    g2 = (d3 @ r(W3)) * dgelu(c["z2"])
    g[ob2:oW3] = g2.sum(0)
    d2 = r(g2)
    g[oW2:ob2] = (d2.T @ c["h1"]).ravel()
    g1 = (d2 @ r(W2)) * dgelu(c["z1"])
    g[ob1:oW2] = g1.sum(0)
    g[oW1:ob1] = (g1.T @ c["x"]).ravel()
    return g, float(np.mean(e * e))
