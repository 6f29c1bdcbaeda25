"""Learned preconditioner: training data from the plain solver, training on
the GPU by the library's own BF16 tensor-core kernels, and evaluation against
Jacobi-PCG at the same tolerance.

Training problems: wellbore meshes whose well pressure is drawn from
U[-30, -5] MPa and friction angle from U[25, 35] deg (seeded), advanced by
Newton to a random load step; their FP32 tangent stays resident in one
library context per problem.  Training pairs: the residual r_k of the plain
(Jacobi) FP32 CG on the Newton right-hand side at iterations k = 0, 64,
128, ... and the remaining solution increment e_k = x_final - x_k.  The loss
of a problem is the log of Kaporin's condition number of M K (M the learned
operator) plus the mean over the drawn pairs of |K e_k - K M r_k|^2 /
|K e_k|^2; its gradient comes from the library (ipfem_learn_grad) and Adam
runs on the library's kernels (ipfem_mlp_adam).
"""
import time

import numpy as np

from . import DEVICE, MIXED, PREC_JACOBI, PREC_MLP, ElastoPlasticIntPointsStructMatrix, WellboreMesh, wellbore_params

SNAPS = list(range(0, 4096, 64))


def _torch():
    import torch

    return torch


def make_solver(n, pw, phi, seed=0, **kw):
    """wellbore n x n in mixed precision with the node grid and a fresh network"""
    wb = WellboreMesh(wellbore_params(n, pw_final=float(pw), phi_deg=float(phi), psi_deg=float(phi), **kw))
    sm = ElastoPlasticIntPointsStructMatrix(wb)
    sm.set_precision(MIXED)
    sm.set_node_grid(2 * n + 1, 2 * n + 1)
    sm.mlp_init(seed)
    return wb, sm


class Problem:
    """one training problem: its context (tangent resident) and its pairs"""

    def __init__(self, wb, sm, R, E, info):
        self.wb, self.sm, self.R, self.E, self.info = wb, sm, R, E, info

    def close(self):
        self.sm.close()
        self.wb.close()


def generate_problems(n=64, n_problems=4, seed=20260101, n_steps=10, cg_rtol=1e-6, snaps=SNAPS, device="cuda"):
    """training problems with (residual, increment) pairs as FP32 device arrays"""
    torch = _torch()
    rng = np.random.default_rng(seed)
    out = []
    for j in range(n_problems):
        pw = float(rng.uniform(-30.0, -5.0))
        phi = float(rng.uniform(25.0, 35.0))
        k = int(rng.integers(1, n_steps + 1))              # load step whose tangent is used
        wb, sm = make_solver(n, pw, phi, seed)
        u = torch.zeros(sm.neq, dtype=torch.float64, device=device)
        if k > 1:
            sm.newton_begin(n_steps, 0, k - 1, newton_max_it=15, cg_rtol=1e-4)
            sm.newton_advance(u, 0, DEVICE)
        sm.SetLoadFactor(k / n_steps)
        R0 = torch.zeros_like(u)
        sm.assemble(u, R0, DEVICE)
        xs = torch.zeros(len(snaps), sm.neq, dtype=torch.float32, device=device)
        rs = torch.zeros_like(xs)
        xf = torch.zeros(sm.neq, dtype=torch.float32, device=device)
        its = sm.cg_snapshots(R0, snaps, xs, rs, xf, rtol=cg_rtol, max_it=60000)
        keep = [i for i, s in enumerate(snaps) if s < its]
        R = rs[keep].contiguous()
        E = (xf[None, :] - xs[keep]).contiguous()
        out.append(Problem(wb, sm, R, E, {"pw": pw, "phi": phi, "step": k, "cg_iters": its, "pairs": len(keep)}))
    return out


def train(problems, steps=300, lr=1e-3, pairs_per_step=8, seed=1, w_kaporin=1.0, w_pairs=1.0):
    """Adam over the problems in turn; returns (parameters, loss per step).
    The first problem's context holds the parameters and the Adam state."""
    torch = _torch()
    rng = np.random.default_rng(seed)
    trainer = problems[0].sm
    losses = []
    for step in range(steps):
        pb = problems[step % len(problems)]
        if pb.sm is not trainer:
            pb.sm.set_mlp_params(trainer.mlp_params())
        npair = pb.R.shape[0]
        idx = torch.tensor(np.sort(rng.choice(npair, size=min(pairs_per_step, npair), replace=False)),
                           device=pb.R.device)
        g, loss = pb.sm.learn_grad(pb.R[idx].contiguous(), pb.E[idx].contiguous(), len(idx), w_kaporin, w_pairs)
        trainer.mlp_adam(g, lr)
        losses.append(loss)
    return trainer.mlp_params(), np.array(losses)


def compare(params, n=400, pw=-12.0, phi=28.0, n_steps=10, newton_iters=6, cg_rtol=1e-4, device="cuda",
            arms=("jacobi", "mlp"), **kw):
    """Runs the same Newton iterations with Jacobi-PCG and with the learned
    FCG (both FP32 inner solves, FP64 Newton); returns per-method statistics."""
    torch = _torch()
    out = {}
    for name, kind in (("jacobi", PREC_JACOBI), ("mlp", PREC_MLP)):
        if name not in arms:
            continue
        wb, sm = make_solver(n, pw, phi, 0, **kw)
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
                     "fallbacks": int(getattr(st, "fcg_fallbacks", 0)),
                     "residuals": log[:, 2].tolist(), "steps": [int(x) for x in log[:, 0]],
                     "cg_per_newton": [int(x) for x in log[:, 1]], "u": u.cpu().numpy()}
        sm.close()
        wb.close()
    return out
