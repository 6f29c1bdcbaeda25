"""CPU oracle of the learned preconditioner (test infrastructure only).

numpy restatement of the per-node network (32 -> 128 -> 128 -> 20), of the
sparse triangular factor G it parameterises and the operator
M = diag(s) G^T G diag(s) (s = sqrt of the Jacobi inverse diagonal, 0 on
Dirichlet dofs), and of the training loss
    L = wk * log(tr(G A^ G^T) / Nf) - wk * (2/Nf) log det G
      + wp * (1/P) sum_p |K e_p - K M r_p|^2 / |K e_p|^2
(A^ = diag(s) K diag(s), Nf free dofs; the first line is the log of Kaporin's
condition number of M K up to a constant) with its parameter gradients.
Every tensor-core operand is rounded to BF16 (round to nearest even) as the
device kernels do; products and sums run in FP64.

Node i = b*gr + a; patch position k = 3*(db+1) + (da+1) for da, db in
{-1, 0, 1}.  G has the blocks k = 0..3 (the lower neighbours) and k = 4 (the
node): G_ik = O_i[4k .. 4k+3] as row-major 2x2 for k < 4 and
G_i4 = [[exp(O_i[16]), 0], [O_i[17], exp(O_i[18])]] with O_i[16], O_i[18]
clamped to [-30, 30]; O_i[19] is unused.
Entries that touch a Dirichlet dof are 0.  Parameter layout of the library:
W1[32][128] b1[128] W2[128][128] b2[128] W3[128][20] b3[20].
"""
import numpy as np

SIZES = [("W1", (32, 128)), ("b1", (128,)), ("W2", (128, 128)), ("b2", (128,)), ("W3", (128, 20)), ("b3", (20,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)
NOUT = 20


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


def factor(gr, gt, O, dinv):
    """G[5][n][2][2] from the network output O[n][20]"""
    nb = neighbours(gr, gt)
    n = gr * gt
    f = (np.asarray(dinv, dtype=np.float64) > 0).astype(np.float64).reshape(n, 2)
    O = np.asarray(O, dtype=np.float64)
    G = np.zeros((5, n, 2, 2))
    for k in range(4):
        ok = nb[:, k] >= 0
        i = np.nonzero(ok)[0]
        j = nb[i, k]
        G[k, i] = O[i, 4 * k:4 * k + 4].reshape(-1, 2, 2) * f[i][:, :, None] * f[j][:, None, :]
    G[4, :, 0, 0] = np.exp(np.clip(O[:, 16], -30.0, 30.0)) * f[:, 0]
    G[4, :, 1, 0] = O[:, 17] * f[:, 1] * f[:, 0]
    G[4, :, 1, 1] = np.exp(np.clip(O[:, 18], -30.0, 30.0)) * f[:, 1]
    return G


def g_mul(gr, gt, G, x):
    """y = G x"""
    nb = neighbours(gr, gt)
    n = gr * gt
    xb = np.asarray(x, dtype=np.float64).reshape(n, 2)
    y = np.zeros((n, 2))
    for k in range(5):
        ok = nb[:, k] >= 0
        y[ok] += np.einsum("ipq,iq->ip", G[k, ok], xb[nb[ok, k]])
    return y.ravel()


def gt_mul(gr, gt, G, y):
    """x = G^T y"""
    nb = neighbours(gr, gt)
    n = gr * gt
    yb = np.asarray(y, dtype=np.float64).reshape(n, 2)
    x = np.zeros((n, 2))
    for k in range(5):
        ok = nb[:, k] >= 0
        i = np.nonzero(ok)[0]
        np.add.at(x, nb[i, k], np.einsum("ipq,ip->iq", G[k, i], yb[i]))
    return x.ravel()


def apply(gr, gt, G, dinv, r):
    """M r = s * G^T (G (s * r))"""
    s = np.sqrt(np.asarray(dinv, dtype=np.float64))
    return s * gt_mul(gr, gt, G, g_mul(gr, gt, G, s * np.asarray(r, dtype=np.float64)))


def kaporin_loss_grad(G, O, Ahat_mul_rows, dinv):
    """log(tr(G A^ G^T)/Nf) - (2/Nf) log det G and its gradient with
    respect to G[5][n][2][2] (the log-det part separately, with respect to
    O[:, 16] and O[:, 18]).  Ahat_mul_rows(G) returns H[5][n][2][2] with
    H_ik[p][q] = (A^ g_ip)[nbr(i, k), q], g_ip row p of G."""
    f = (np.asarray(dinv) > 0).astype(np.float64).reshape(-1, 2)
    nf = f.sum()
    H = Ahat_mul_rows(G)
    T = float((G * H).sum())
    loss = np.log(T / nf) - 2.0 / nf * float((O[:, 16] * f[:, 0]).sum() + (O[:, 18] * f[:, 1]).sum())
    dG = 2.0 / T * H
    dlogdet = np.zeros((O.shape[0], 2))
    dlogdet[:, 0] = -2.0 / nf * f[:, 0]
    dlogdet[:, 1] = -2.0 / nf * f[:, 1]
    return loss, dG, dlogdet


def dO_from_dG(O, dG, dinv, gr, gt, dlogdet=None):
    """chain rule G(O) -> dL/dO[n][20]"""
    nb = neighbours(gr, gt)
    n = O.shape[0]
    f = (np.asarray(dinv) > 0).astype(np.float64).reshape(n, 2)
    dO = np.zeros((n, NOUT))
    for k in range(4):
        ok = nb[:, k] >= 0
        i = np.nonzero(ok)[0]
        j = nb[i, k]
        dO[i, 4 * k:4 * k + 4] = (dG[k, i] * f[i][:, :, None] * f[j][:, None, :]).reshape(-1, 4)
    in16 = (np.abs(O[:, 16]) < 30.0).astype(np.float64)
    in18 = (np.abs(O[:, 18]) < 30.0).astype(np.float64)
    dO[:, 16] = dG[4, :, 0, 0] * np.exp(O[:, 16]) * f[:, 0] * in16
    dO[:, 17] = dG[4, :, 1, 0] * f[:, 1] * f[:, 0]
    dO[:, 18] = dG[4, :, 1, 1] * np.exp(O[:, 18]) * f[:, 1] * in18
    if dlogdet is not None:
        dO[:, 16] += dlogdet[:, 0] * in16
        dO[:, 18] += dlogdet[:, 1] * in18
    return dO


def pair_loss_grad(G, matvec, gr, gt, dinv, R, E):
    """(1/P) sum_p |K e_p - K M r_p|^2 / |K e_p|^2 and its gradient w.r.t. G"""
    nb = neighbours(gr, gt)
    n = gr * gt
    s = np.sqrt(np.asarray(dinv, dtype=np.float64))
    npair = len(R)
    dG = np.zeros_like(G)
    loss = 0.0
    for r, e in zip(R, E):
        r = np.asarray(r, dtype=np.float64)
        ae = matvec(np.asarray(e, dtype=np.float64))
        rh = s * r
        y = g_mul(gr, gt, G, rh)
        z = s * gt_mul(gr, gt, G, y)
        res = ae - matvec(z)
        aa = ae @ ae
        if not aa > 0:
            continue
        loss += (res @ res) / aa / npair
        u = s * (-2.0 / (aa * npair)) * matvec(res)        # dL/d(G^T y) premultiplied by s
        v = g_mul(gr, gt, G, u)
        yb, ub, vb, rb = y.reshape(n, 2), u.reshape(n, 2), v.reshape(n, 2), rh.reshape(n, 2)
        for k in range(5):
            i = np.nonzero(nb[:, k] >= 0)[0]
            j = nb[i, k]
            dG[k, i] += yb[i][:, :, None] * ub[j][:, None, :] + vb[i][:, :, None] * rb[j][:, None, :]
    return loss, dG


def ahat_rows(gr, gt, blocks, dinv):
    """Ahat_mul_rows for the 5-node lower patches: blocks(j, l) returns the
    2x2 tangent block K_jl (zeros if absent)"""
    nb = neighbours(gr, gt)
    n = gr * gt
    s = np.sqrt(np.asarray(dinv, dtype=np.float64)).reshape(n, 2)

    def mul(G):
        H = np.zeros_like(G)
        for i in range(n):
            for k in range(5):
                jk = nb[i, k]
                if jk < 0:
                    continue
                for l in range(5):
                    jl = nb[i, l]
                    if jl < 0:
                        continue
                    Ah = s[jk][:, None] * blocks(jk, jl) * s[jl][None, :]
                    # H_ik[p][q] += sum_t Ahat[jk q][jl t] G_il[p][t]
                    H[k, i] += G[l, i] @ Ah.T
        return H
    return mul


def loss_grad_O(O, matvec, blocks, gr, gt, dinv, R, E, wk=1.0, wp=1.0):
    """the combined loss and dL/dO[n][20]"""
    G = factor(gr, gt, O, dinv)
    lk, dGk, dld = kaporin_loss_grad(G, O, ahat_rows(gr, gt, blocks, dinv), dinv)
    loss, dG, dlogdet = wk * lk, wk * dGk, wk * dld
    if wp > 0 and len(R):
        lp, dGp = pair_loss_grad(G, matvec, gr, gt, dinv, R, E)
        loss += wp * lp
        dG = dG + wp * dGp
    return loss, dO_from_dG(O, dG, dinv, gr, gt, dlogdet)


def loss_and_grads(p, X, matvec, blocks, gr, gt, dinv, R, E, wk=1.0, wp=1.0):
    """loss and parameter gradient (packed)"""
    P = unpack(p)
    O, (X, H1, H2) = forward(p, X)
    loss, dO = loss_grad_O(O, matvec, blocks, gr, gt, dinv, R, E, wk, wp)
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
