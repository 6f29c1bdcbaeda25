"""Learned preconditioner: training data from the plain solver, training on
the GPU by the library's own BF16 tensor-core kernels, and evaluation against
Jacobi-PCG at the same tolerance.

Training pairs (per node): the residual r_k of the plain (Jacobi) FP32 CG at
iterations k = 0, 32, 64, ..., 2048 and the remaining solution increment
e_k = x_final - x_k, for Newton residuals of wellbore problems whose well
pressure is drawn from U[-30, -5] MPa and friction angle from U[25, 35] deg
(seeded).  The network input is the 32-feature vector of the node (computed
from r_k by the library), the target is e_k / (s * Dinv) so that the network
output is dimensionless (z = (own + output) * s * Dinv).
"""
import time

import numpy as np

from . import (DEVICE, MIXED, PREC_JACOBI, PREC_MLP, ElastoPlasticIntPointsStructMatrix, WellboreMesh,
               wellbore_params)

SNAPS = [0, 32, 64, 96, 128, 160, 256, 288, 512, 544, 1024, 1056, 2048, 2080]


def _torch():
    import torch

    return torch


def make_solver(n, pw, phi, seed=0, n_steps=10):
    wb = WellboreMesh(wellbore_params(n, pw_final=float(pw), phi_deg=float(phi), psi_deg=float(phi)))
    sm = ElastoPlasticIntPointsStructMatrix(wb)
    sm.set_precision(MIXED)
    sm.set_node_grid(2 * n + 1, 2 * n + 1)
    sm.mlp_init(seed)
    return wb, sm


def generate_training_data(n=400, n_samples=50000, n_problems=8, seed=20260101, n_steps=10, cg_rtol=1e-5,
                           target="increment", s_floor=1e-2, t_cap=100.0, device="cuda"):
    """Returns (X [samples, 32], Y [samples, 2]) as FP32 device tensors.

    target "increment": the CG solution increment over the next 32 iterations,
    x_{k+32} - x_k, for the residual r_k; "error": the remaining increment
    x_final - x_k.  Samples whose patch residual scale s is below s_floor times
    the RMS scale of the snapshot, or whose scaled target exceeds t_cap, are
    dropped (the residual there carries no information about the increment)."""
    torch = _torch()
    rng = np.random.default_rng(seed)
    Xs, Ys = [], []
    per_problem = n_samples // n_problems
    for j in range(n_problems):
        pw = rng.uniform(-30.0, -5.0)
        phi = rng.uniform(25.0, 35.0)
        wb, sm = make_solver(n, pw, phi, seed, n_steps)
        u = torch.zeros(sm.neq, dtype=torch.float64, device=device)
        k = int(rng.integers(1, n_steps + 1))              # load steps already applied
        if k > 1:
            sm.newton_begin(n_steps, 0, k - 1, newton_max_it=15, cg_rtol=1e-4)
            sm.newton_advance(u, 0, DEVICE)
        sm.SetLoadFactor(k / n_steps)
        R = torch.zeros_like(u)
        sm.assemble(u, R, DEVICE)
        xs = torch.zeros(len(SNAPS), sm.neq, dtype=torch.float32, device=device)
        rs = torch.zeros_like(xs)
        xf = torch.zeros(sm.neq, dtype=torch.float32, device=device)
        its = sm.cg_snapshots(R, SNAPS, xs, rs, xf, rtol=cg_rtol, max_it=60000)
        snaps = [i for i, s in enumerate(SNAPS) if s < its]
        X = torch.zeros(sm.n_nodes, 32, dtype=torch.float32, device=device)
        S = torch.zeros(sm.n_nodes, dtype=torch.float32, device=device)
        T = torch.zeros(sm.neq, dtype=torch.float32, device=device)
        fixed = torch.tensor(wb.array("fixed").reshape(-1, 2).min(axis=1) == 0, device=device)
        free_nodes_t = torch.nonzero(fixed).flatten()
        for si in snaps:
            if target == "increment":
                nxt = SNAPS[si] + 32
                if nxt >= its:
                    continue
                xn = xs[SNAPS.index(nxt)] if nxt in SNAPS else None
                if xn is None:
                    continue
                e = xn - xs[si]
            else:
                e = xf - xs[si]
            sm.mlp_features(rs[si].double(), X, S)
            sm.mlp_targets(e, S, T)
            Tn = T.view(-1, 2)
            srms = torch.sqrt((S[free_nodes_t] ** 2).mean())
            good = (S > s_floor * srms) & (Tn.abs().max(dim=1).values < t_cap) & torch.isfinite(Tn).all(dim=1)
            good[~fixed] = False
            cand = torch.nonzero(good).flatten().cpu().numpy()
            if len(cand) == 0:
                continue
            pick = rng.choice(cand, size=min(len(cand), per_problem // len(snaps)), replace=False)
            idx = torch.tensor(pick, device=device)
            Xs.append(X[idx].clone())
            Ys.append(Tn[idx].clone())
        sm.close()
        wb.close()
    X = torch.cat(Xs)
    Y = torch.cat(Ys)
    ok = torch.isfinite(Y).all(dim=1) & torch.isfinite(X).all(dim=1)
    return X[ok].contiguous(), Y[ok].contiguous()


def train(X, Y, epochs=40, batch=2048, lr=2e-3, seed=1, n_host=8):
    """Trains a fresh network on (X, Y) with the library's kernels; returns
    (parameters as a numpy FP32 vector, loss per epoch)."""
    wb, sm = make_solver(n_host, -10.0, 30.0, seed)
    losses = sm.mlp_train(X, Y, X.shape[0], epochs=epochs, batch=batch, lr=lr, seed=seed)
    p = sm.mlp_params()
    sm.close()
    wb.close()
    return p, losses


def compare(params, n=400, pw=-12.0, phi=28.0, n_steps=10, newton_iters=6, cg_rtol=1e-4, device="cuda"):
    """Runs the same Newton iterations with Jacobi-PCG and with the learned
    FCG (both FP32 inner solves, FP64 Newton); returns per-method statistics."""
    torch = _torch()
    out = {}
    for name, kind in (("jacobi", PREC_JACOBI), ("mlp", PREC_MLP)):
        wb, sm = make_solver(n, pw, phi, 0, n_steps)
        sm.set_mlp_params(params)
        sm.set_preconditioner(kind)
        u = torch.zeros(sm.neq, dtype=torch.float64, device=device)
        sm.newton_begin(n_steps, newton_max_it=40, cg_rtol=cg_rtol)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st, log = sm.newton_advance(u, newton_iters, DEVICE)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out[name] = {"newton_iters": st.newton_iters, "cg_iters": int(st.cg_iters),
                     "ms_per_newton": 1e3 * dt / max(1, st.newton_iters), "ms_solve": st.ms_solve,
                     "residuals": log[:, 2].tolist(), "u": u.cpu().numpy()}
        sm.close()
        wb.close()
    return out
