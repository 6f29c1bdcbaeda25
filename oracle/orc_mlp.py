"""CPU oracle of the learned preconditioner (test infrastructure only).

numpy restatement of the per-node network (32 -> 128 -> 128 -> 36), of the
symmetric 3x3-patch operator it parameterises, and of the training loss
L = (1/P) sum_p |K e_p - K M r_p|^2 / |K e_p|^2 with its parameter gradients.
Every tensor-core operand is rounded to BF16 (round to nearest even) as the
device kernels do; products and sums run in FP64.

Parameter layout of the library: W1[32][128] b1[128] W2[128][128] b2[128]
W3[128][36] b3[36].  Node i = b*gr + a; patch position k = 3*(db+1) + (da+1),
k = 4 the node itself, 8 - k the mirror position.
"""
import numpy as np

SIZES = [("W1", (32, 128)), ("b1", (128,)), ("W2", (128, 128)), ("b2", (128,)), ("W3", (128, 36)), ("b3", (36,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)


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


def neighbours(gr, gt):
    """nb[n][9]: node at each patch position, -1 outside the grid"""
    n = gr * gt
    i = np.arange(n)
    a, b = i % gr, i // gr
    nb = -np.ones((n, 9), dtype=np.int64)
    for k in range(9):
        aa, bb = a + k % 3 - 1, b + k // 3 - 1
        ok = (aa >= 0) & (bb >= 0) & (aa < gr) & (bb < gt)
        nb[ok, k] = bb[ok] * gr + aa[ok]
    return nb


def features(gr, gt, row_ptr, col, K, dinv):
    """X[n][32] from the block tangent (CSR of 2x2 blocks K[n_blocks][2][2])
    and the Jacobi inverse diagonal (0 on Dirichlet dofs)"""
    nb = neighbours(gr, gt)
    n = gr * gt
    s = np.sqrt(np.asarray(dinv, dtype=np.float64)).reshape(n, 2)
    X = np.zeros((n, 32))
    for i in range(n):
        cols = col[row_ptr[i]:row_ptr[i + 1]]
        m = 0
        for k in range(9):
            if k == 4:
                continue
            j = nb[i, k]
            if j >= 0:
                t = np.searchsorted(cols, j)
                if t < len(cols) and cols[t] == j:
                    blk = K[row_ptr[i] + t]
                    X[i, 4 * m:4 * m + 4] = (s[i][:, None] * blk * s[j][None, :]).ravel()
            m += 1
    return X


def forward(p, X):
    """network output O[rows][36] and the hidden layers"""
    P = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    H1 = np.maximum(bf16(X) @ bf16(P["W1"]) + P["b1"], 0.0)
    H2 = np.maximum(bf16(H1) @ bf16(P["W2"]) + P["b2"], 0.0)
    O = bf16(H2) @ bf16(P["W3"]) + P["b3"]
    return O, (X, H1, H2)


def operator(gr, gt, O, dinv):
    """M[9][n][2][2] = s_i ((O_ik + O_j(8-k)^T)/2 + [k == 4] I) s_j"""
    nb = neighbours(gr, gt)
    n = gr * gt
    s = np.sqrt(np.asarray(dinv, dtype=np.float64)).reshape(n, 2)
    Ob = np.asarray(O, dtype=np.float64).reshape(n, 9, 2, 2)
    M = np.zeros((9, n, 2, 2))
    for k in range(9):
        ok = nb[:, k] >= 0
        i = np.nonzero(ok)[0]
        j = nb[i, k]
        mh = 0.5 * (Ob[i, k] + np.transpose(Ob[j, 8 - k], (0, 2, 1)))
        if k == 4:
            mh = mh + np.eye(2)
        M[k, i] = s[i][:, :, None] * mh * s[j][:, None, :]
    return M


def apply(gr, gt, M, r):
    nb = neighbours(gr, gt)
    n = gr * gt
    rb = np.asarray(r, dtype=np.float64).reshape(n, 2)
    z = np.zeros((n, 2))
    for k in range(9):
        ok = nb[:, k] >= 0
        z[ok] += np.einsum("ipq,iq->ip", M[k, ok], rb[nb[ok, k]])
    return z.ravel()


def patch_loss_grad(O, matvec, gr, gt, dinv, R, E):
    """loss L = (1/P) sum_p |K e_p - K M r_p|^2 / |K e_p|^2 of the operator
    built from O[n][36] and dL/dO[n][36]"""
    n = gr * gt
    M = operator(gr, gt, O, dinv)
    nb = neighbours(gr, gt)
    s = np.sqrt(np.asarray(dinv, dtype=np.float64)).reshape(n, 2)
    npair = len(R)
    dO = np.zeros((n, 9, 2, 2))
    loss = 0.0
    for r, e in zip(R, E):
        r = np.asarray(r, dtype=np.float64)
        ae = matvec(np.asarray(e, dtype=np.float64))
        az = matvec(apply(gr, gt, M, r))
        res = ae - az
        aa = ae @ ae
        if not aa > 0:
            continue
        loss += (res @ res) / aa / npair
        g = matvec(res)
        c = -1.0 / (aa * npair)
        rh = s * r.reshape(n, 2)
        gh = s * g.reshape(n, 2)
        for k in range(9):
            i = np.nonzero(nb[:, k] >= 0)[0]
            j = nb[i, k]
            dO[i, k] += c * (gh[i][:, :, None] * rh[j][:, None, :] + rh[i][:, :, None] * gh[j][:, None, :])
    return loss, dO.reshape(n, 36)


def loss_and_grads(p, X, matvec, gr, gt, dinv, R, E):
    """loss and parameter gradient (packed) for pairs R[P][neq], E[P][neq];
    matvec(v) applies the symmetric tangent (Dirichlet rows and columns 0)"""
    P = unpack(p)
    O, (X, H1, H2) = forward(p, X)
    loss, dO = patch_loss_grad(O, matvec, gr, gt, dinv, R, E)
    grads = {}
    grads["W3"] = bf16(H2).T @ bf16(dO)
    grads["b3"] = dO.sum(0)
    dH2 = (bf16(dO) @ bf16(P["W3"]).T) * (H2 > 0)
    grads["W2"] = bf16(H1).T @ bf16(dH2)
    grads["b2"] = dH2.sum(0)
    dH1 = (bf16(dH2) @ bf16(P["W2"]).T) * (H1 > 0)
    grads["W1"] = bf16(X).T @ bf16(dH1)
    grads["b1"] = dH1.sum(0)
    return loss, pack(grads)
