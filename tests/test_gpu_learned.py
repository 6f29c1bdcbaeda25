"""Learned preconditioner: tensor-core forward and gradients against the CPU
oracle (oracle/orc_mlp.py), FCG with the untrained network equals Jacobi,
training on the GPU, and what the trained network gains over Jacobi-PCG."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ip = pytest.importorskip("intpointsfem_gb300")
torch = pytest.importorskip("torch")
from intpointsfem_gb300 import learned  # noqa: E402
from oracle import orc_mlp  # noqa: E402


def _host():
    wb, sm = learned.make_solver(8, -10.0, 30.0, seed=3)
    return wb, sm


def _random_params(rng, scale3=0.2):
    d = {"W1": rng.normal(size=(32, 128)) * np.sqrt(2 / 32), "b1": rng.normal(size=128) * 0.1,
         "W2": rng.normal(size=(128, 128)) * np.sqrt(2 / 128), "b2": rng.normal(size=128) * 0.1,
         "W3": rng.normal(size=(128, 2)) * scale3, "b3": rng.normal(size=2) * 0.1}
    return orc_mlp.pack(d)


def test_forward_matches_cpu_oracle():
    rng = np.random.default_rng(0)
    wb, sm = _host()
    p = _random_params(rng)
    sm.set_mlp_params(p)
    X = rng.normal(size=(1000, 32)).astype(np.float32)
    dX = torch.tensor(X, device="cuda")
    dO = torch.zeros(1000, 2, device="cuda")
    sm.mlp_forward(dX, 1000, dO)
    O_ref, _ = orc_mlp.forward(sm.mlp_params(), X)
    O = dO.cpu().numpy()
    err = np.abs(O - O_ref).max() / np.abs(O_ref).max()
    assert err < 2e-3, err


def test_gradients_match_cpu_oracle():
    rng = np.random.default_rng(1)
    wb, sm = _host()
    p = _random_params(rng)
    sm.set_mlp_params(p)
    n = 3000
    X = rng.normal(size=(n, 32)).astype(np.float32)
    Y = rng.normal(size=(n, 2)).astype(np.float32)
    g, loss = sm.mlp_grad(torch.tensor(X, device="cuda"), torch.tensor(Y, device="cuda"), n)
    loss_ref, g_ref = orc_mlp.loss_and_grads(sm.mlp_params(), X, Y)
    assert loss == pytest.approx(loss_ref, rel=2e-3)
    gd, rd = orc_mlp.unpack(g), orc_mlp.unpack(g_ref)
    for name, _ in orc_mlp.SIZES:
        e = np.linalg.norm(gd[name] - rd[name]) / np.linalg.norm(rd[name])
        assert e < 1e-2, (name, e)


def test_untrained_network_is_jacobi_inside_fcg():
    """W3 = 0 at initialisation: the preconditioner is Jacobi, so FCG and
    Jacobi-PCG take the same number of iterations to the same tolerance."""
    wb, sm = learned.make_solver(32, -10.0, 30.0, seed=0)
    u = torch.zeros(sm.neq, dtype=torch.float64, device="cuda")
    R = torch.zeros_like(u)
    sm.SetLoadFactor(0.5)
    sm.assemble(u, R, ip.DEVICE)
    x0, it0 = sm.solve(R, torch.zeros_like(u), rtol=1e-5, where=ip.DEVICE)
    sm.set_preconditioner(ip.PREC_MLP)
    x1, it1 = sm.solve(R, torch.zeros_like(u), rtol=1e-5, where=ip.DEVICE)
    assert abs(it1 - it0) <= max(3, it0 // 20), (it0, it1)
    assert torch.allclose(x0, x1, rtol=1e-3, atol=1e-3 * float(x0.abs().max()))


def test_training_and_gain_over_jacobi():
    """Small wellbore (48 x 48): data from the plain solver, training on the
    GPU, then the same Newton iterations with Jacobi-PCG and with the learned
    FCG.  Both must reach the same Newton tolerance; the gain (CG iterations
    and solve time) is reported."""
    X, Y = learned.generate_training_data(n=48, n_samples=16000, n_problems=4, seed=11)
    assert X.shape[0] > 8000
    p, losses = learned.train(X, Y, epochs=25, batch=1024, lr=2e-3, seed=2)
    assert np.isfinite(losses).all() and losses[-1] < losses[0]
    res = learned.compare(p, n=48, pw=-12.0, phi=28.0, newton_iters=6)
    j, m = res["jacobi"], res["mlp"]
    print("learned vs Jacobi (48x48): CG iterations %d vs %d, solve ms %.1f vs %.1f, loss %.3g -> %.3g"
          % (m["cg_iters"], j["cg_iters"], m["ms_solve"], j["ms_solve"], losses[0], losses[-1]))
    assert m["newton_iters"] == j["newton_iters"]
    # both Newton sequences reach the same displacement to the Newton tolerance
    du = np.abs(m["u"] - j["u"]).max() / np.abs(j["u"]).max()
    assert du < 1e-4, du
