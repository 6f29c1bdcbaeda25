"""CPU oracle of the learned preconditioner's network (test infrastructure only).

numpy restatement of the forward pass and of the gradients of the MSE loss,
with every tensor-core operand rounded to BF16 (round to nearest even) as the
device kernels do, products and sums in FP64.  Parameter layout of the
library: W1[32][128] b1[128] W2[128][128] b2[128] W3[128][2] b3[2]; the
output has a skip connection from input features 8 and 9.
"""
import numpy as np

SIZES = [("W1", (32, 128)), ("b1", (128,)), ("W2", (128, 128)), ("b2", (128,)), ("W3", (128, 2)), ("b3", (2,))]


def unpack(p):
    out, o = {}, 0
    for name, shp in SIZES:
        n = int(np.prod(shp))
        out[name] = np.asarray(p[o:o + n], dtype=np.float64).reshape(shp)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float32).ravel() for name, _ in SIZES])


def bf16(x):
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((u >> 16) & 1) + np.uint32(0x7FFF)
    return ((u + r) & np.uint32(0xFFFF0000)).view(np.float32).astype(np.float64)


def forward(p, X):
    P = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    H1 = np.maximum(bf16(X) @ bf16(P["W1"]) + P["b1"], 0.0)
    H2 = np.maximum(bf16(H1) @ bf16(P["W2"]) + P["b2"], 0.0)
    O = X[:, 8:10] + bf16(H2) @ bf16(P["W3"]) + P["b3"]
    return O, (X, H1, H2)


def loss_and_grads(p, X, Y):
    P = unpack(p)
    O, (X, H1, H2) = forward(p, X)
    n = X.shape[0]
    E = O - np.asarray(Y, dtype=np.float64)
    loss = float((E * E).sum() / n)
    dO = 2.0 * E / n
    g = {}
    g["W3"] = bf16(H2).T @ bf16(dO)
    g["b3"] = dO.sum(0)
    dH2 = (dO @ bf16(P["W3"]).T) * (H2 > 0)
    g["W2"] = bf16(H1).T @ bf16(dH2)
    g["b2"] = dH2.sum(0)
    dH1 = (bf16(dH2) @ bf16(P["W2"]).T) * (H1 > 0)
    g["W1"] = bf16(X).T @ bf16(dH1)
    g["b1"] = dH1.sum(0)
    return loss, pack(g)
