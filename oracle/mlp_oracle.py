"""CPU oracle of the surrogate MLP -- test infrastructure only.

FP64 forward and backward of 8 -> 4 x 256 GELU (tanh form) -> 4 with BF16 rounding
emulated at exactly the points where the GPU kernels round
(bldfm_gb300/csrc/surrogate.cu): hidden weights as BF16, the activations of
the first three hidden layers and every GELU'(Z) stored as BF16 (the last
hidden layer stays FP32), and every dZ rounded to BF16 before it enters a
GEMM.  Accumulations are FP64 here and FP32 on the GPU; tanh is exact here
and the hardware tanh.approx there.
"""

import math

import numpy as np

H, N_IN, N_OUT = 256, 8, 4


def bf16(x):
    """Round to BF16 (nearest-even) and return as float64."""
    u = np.ascontiguousarray(np.asarray(x, dtype=np.float32)).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


GELU_C, GELU_A = math.sqrt(2.0 / math.pi), 0.044715


def gelu(z):
    """GELU in its tanh form (Hendrycks & Gimpel, 2016), as the kernels use it."""
    return 0.5 * z * (1.0 + np.tanh(GELU_C * (z + GELU_A * z**3)))


def gelu_d(z):
    t = np.tanh(GELU_C * (z + GELU_A * z**3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * GELU_C * (1.0 + 3.0 * GELU_A * z * z)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W0 = p[o : o + N_IN * H].reshape(N_IN, H)
    o += N_IN * H
    b0 = p[o : o + H]
    o += H
    Wt, b = [], []
    for _ in range(3):
        Wt.append(p[o : o + H * H].reshape(H, H))
        o += H * H
        b.append(p[o : o + H])
        o += H
    W4 = p[o : o + H * N_OUT].reshape(H, N_OUT)
    o += H * N_OUT
    b4 = p[o : o + N_OUT]
    return W0, b0, Wt, b, W4, b4


def forward_backward(p, X, T, w):
    """Returns (Y, loss, grad flat) for inputs X [n][8], targets T [n][4], weights w [n][4]."""
    W0, b0, Wt, b, W4, b4 = unpack(p)
    X = np.asarray(X, dtype=np.float64)[:, :N_IN]
    n = X.shape[0]
    Wtb = [bf16(m) for m in Wt]
    z = X @ W0 + b0
    Hs = [bf16(gelu(z))]
    Gs = [bf16(gelu_d(z))]
    for j in range(3):
        z = Hs[-1] @ Wtb[j].T + b[j]
        Hs.append(bf16(gelu(z)) if j < 2 else gelu(z))
        Gs.append(bf16(gelu_d(z)))
    Y = Hs[3] @ W4 + b4
    e = Y - T
    w = np.asarray(w, dtype=np.float64).reshape(n, N_OUT)
    loss = float(np.sum(w * e * e) / n)
    dY = 2.0 * w * e / n
    g = {}
    g["W4"] = Hs[3].T @ dY
    g["b4"] = dY.sum(0)
    dZ = bf16((dY @ W4.T) * Gs[3])
    for j in (2, 1, 0):
        g["b%d" % (j + 1)] = dZ.sum(0)
        g["Wt%d" % (j + 1)] = dZ.T @ Hs[j]
        dZ = bf16((dZ @ Wtb[j]) * Gs[j])
    g["b0"] = dZ.sum(0)
    g["W0"] = X.T @ dZ
    flat = np.concatenate(
        [g["W0"].ravel(), g["b0"]]
        + sum([[g["Wt%d" % j].ravel(), g["b%d" % j]] for j in (1, 2, 3)], [])
        + [g["W4"].ravel(), g["b4"]]
    )
    return Y, loss, flat
