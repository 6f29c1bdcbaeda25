"""Train the learned patch preconditioner on the GPU and write its weights.

    python -m intpointsfem_gb300.train_preconditioner --n 400 --problems 4 --steps 400 \\
        --out intpointsfem_gb300/weights/patch_net.npy

Problems: n x n wellbore meshes with well pressure U[-30, -5] MPa and
friction angle U[25, 35] deg (seeded), each advanced by Newton to a random
load step; pairs: (residual, solution increment) snapshots of the plain FP32
Jacobi-CG on the Newton right-hand side (learned.generate_problems).  The
gradient pass and Adam run on the library's kernels.  The report (JSON beside
the weights) records the data, the loss curve and, for held-out problems, the
CG iterations and solve times of Jacobi-PCG and of the learned FCG over the
same Newton iterations.
"""
import argparse
import json
import os
import time

import numpy as np

from . import learned

WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "patch_net.npy")


def load_weights(path=WEIGHTS):
    """the shipped network parameters (FP32, 23316 values)"""
    return np.load(path).astype(np.float32)


def evaluate(params, n, newton_iters, cases=((-12.0, 28.0), (-25.0, 33.0)), **kw):
    """Jacobi-PCG vs learned FCG over the same Newton iterations of held-out problems"""
    out = []
    for pw, phi in cases:
        res = learned.compare(params, n=n, pw=pw, phi=phi, newton_iters=newton_iters, **kw)
        j, m = res["jacobi"], res["mlp"]
        out.append({"n": n, "pw": pw, "phi": phi, "newton_iters": m["newton_iters"],
                    "cg_iters_jacobi": j["cg_iters"], "cg_iters_learned": m["cg_iters"],
                    "ms_solve_jacobi": j["ms_solve"], "ms_solve_learned": m["ms_solve"],
                    "fallbacks": m["fallbacks"],
                    "load_steps_jacobi": j["steps"], "load_steps_learned": m["steps"],
                    "cg_per_newton_jacobi": j["cg_per_newton"], "cg_per_newton_learned": m["cg_per_newton"],
                    "max_rel_du": float(np.abs(m["u"] - j["u"]).max() / np.abs(j["u"]).max())})
    return out


def time_step(n, pairs, steps, warmup=2):
    """ms per training step (gradient pass + Adam on the device gradient) on an
    n x n problem, pairs of random FP32 vectors; CUDA events on the library's
    stream after `warmup` untimed gradient passes"""
    import torch
    import intpointsfem_gb300 as ip
    wb, sm = learned.make_solver(n, -10.0, 30.0, seed=3)
    try:
        u = torch.zeros(sm.neq, dtype=torch.float64, device="cuda")
        sm.SetLoadFactor(0.5)
        R = torch.zeros_like(u)
        sm.assemble(u, R, ip.DEVICE)
        g = torch.Generator(device="cuda").manual_seed(5)
        r = torch.randn(pairs, sm.neq, device="cuda", dtype=torch.float32, generator=g)
        e = torch.randn(pairs, sm.neq, device="cuda", dtype=torch.float32, generator=g)
        for _ in range(warmup):
            sm.learn_grad(r, e, pairs, 1.0, 1.0)
        torch.cuda.synchronize()
        st = torch.cuda.ExternalStream(sm.stream, device=u.device)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(st)
        for _ in range(steps):
            sm.learn_grad(r, e, pairs, 1.0, 1.0)
            sm.mlp_adam(None, 1e-5)
        t1.record(st)
        torch.cuda.synchronize()
        return t0.elapsed_time(t1) / steps
    finally:
        sm.close()
        wb.close()


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=400)
    ap.add_argument("--problems", type=int, default=4)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--pairs-per-step", type=int, default=8)
    ap.add_argument("--seed", type=int, default=20260101)
    ap.add_argument("--eval-n", type=int, default=0, help="mesh of the held-out comparison (0: --n)")
    ap.add_argument("--eval-newton", type=int, default=4)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--eval-only", default="", help="evaluate these weights instead of training")
    ap.add_argument("--material-mode", type=int, default=0, help="0 uniform, 1 lognormal cohesion, 2 + friction angle")
    ap.add_argument("--c-cv", type=float, default=0.2)
    ap.add_argument("--n-steps", type=int, default=10)
    ap.add_argument("--learned-only", action="store_true",
                    help="with --eval-only: run only the learned arm of the first case (profiling)")
    ap.add_argument("--time-step", type=int, default=0,
                    help="time this many gradient + Adam steps on one --n problem with random pairs and exit")
    a = ap.parse_args(argv)
    if a.time_step:
        print("ms per Adam step (%dx%d, %d pairs): %.2f" % (a.n, a.n, a.pairs_per_step,
                                                            time_step(a.n, a.pairs_per_step, a.time_step)),
              flush=True)
        return
    mat = {"material_mode": a.material_mode, "c_cv": a.c_cv} if a.material_mode else {}
    if a.eval_only and a.learned_only:
        res = learned.compare(load_weights(a.eval_only), n=a.eval_n or a.n, newton_iters=a.eval_newton,
                              n_steps=a.n_steps, arms=("mlp",), **mat)["mlp"]
        print("learned", json.dumps({k: v for k, v in res.items() if k != "u"}), flush=True)
        return
    if a.eval_only:
        params = load_weights(a.eval_only)
        for row in evaluate(params, a.eval_n or a.n, a.eval_newton, n_steps=a.n_steps, **mat):
            print("eval", json.dumps(row), flush=True)
        return
    t0 = time.time()
    probs = learned.generate_problems(n=a.n, n_problems=a.problems, seed=a.seed)
    t_data = time.time() - t0
    info = [pb.info for pb in probs]
    n_pairs = sum(pb.R.shape[0] for pb in probs)
    neq = probs[0].sm.neq
    print("data: %d problems, %d (residual, increment) pairs of %d dofs, %.1f s" % (len(probs), n_pairs, neq, t_data),
          flush=True)
    t0 = time.time()
    try:
        params, losses = learned.train(probs, steps=a.steps, lr=a.lr, pairs_per_step=a.pairs_per_step,
                                       seed=a.seed + 1)
    finally:
        for pb in probs:
            pb.close()
    t_train = time.time() - t0
    print("train: %d Adam steps, %.1f s, loss %.4g -> %.4g" % (a.steps, t_train, losses[:5].mean(),
                                                                losses[-20:].mean()), flush=True)
    os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
    np.save(a.out, params.astype(np.float32))
    ev = evaluate(params, a.eval_n or a.n, a.eval_newton)
    for row in ev:
        print("eval", json.dumps(row), flush=True)
    report = {"n": a.n, "problems": info, "pairs": n_pairs, "dofs_per_pair": neq, "steps": a.steps, "lr": a.lr,
              "pairs_per_step": a.pairs_per_step, "seconds_data": t_data, "seconds_train": t_train,
              "loss_first5": float(losses[:5].mean()), "loss_last20": float(losses[-20:].mean()),
              "loss": [float(x) for x in losses[::10]], "eval": ev}
    with open(os.path.splitext(a.out)[0] + ".json", "w") as f:
        json.dump(report, f, indent=1)


if __name__ == "__main__":
    main()
