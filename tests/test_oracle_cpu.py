"""CPU checks of the oracle's assembly and solver (the properties the GPU
parity tests rely on)."""
import contextlib

import numpy as np
import pytest

from oracle import pyoracle as po


@pytest.fixture(scope="module")
def P8():
    return po.OracleProblem(po.default_params(8), nthreads=2)


def test_in_situ_state_is_in_discrete_equilibrium(P8):
    r = P8.assemble_residual(np.zeros(P8.neq), 0.0)
    assert np.abs(r).max() < 1e-10 * np.abs(P8.arr("f0")).max()


def test_dot_tree_matches_numpy_and_partials():
    rng = np.random.default_rng(1)
    for nn in (1, 31, 256, 257, 5000):
        a, b = rng.normal(size=2 * nn), rng.normal(size=2 * nn)
        d = po.dot(a, b)
        assert d == pytest.approx(float(np.dot(a, b)), rel=1e-13, abs=1e-13)
    # exact for integers (any order)
    a = np.arange(2000, dtype=np.float64)
    assert po.dot(a, a) == float(np.dot(a, a))


def test_tangent_matches_finite_differences_in_elastic_state(P8):
    rng = np.random.default_rng(0)
    fixed = P8.arr("fixed").astype(bool)
    u = np.zeros(P8.neq)
    P8.assemble(u, 0.3)
    v = rng.normal(size=P8.neq)
    v[fixed] = 0
    Kv = P8.spmv(v)
    h = 1e-9
    fd = -(P8.assemble_residual(u + h * v, 0.3) - P8.assemble_residual(u - h * v, 0.3)) / (2 * h)
    assert np.linalg.norm(Kv - fd) / np.linalg.norm(fd) < 1e-6


def test_tangent_is_symmetric_and_fixed_rows_masked(P8):
    P8.assemble(np.zeros(P8.neq), 0.2)
    rng = np.random.default_rng(3)
    fixed = P8.arr("fixed").astype(bool)
    x, y = rng.normal(size=P8.neq), rng.normal(size=P8.neq)
    x[fixed] = 0
    y[fixed] = 0
    assert np.dot(y, P8.spmv(x)) == pytest.approx(np.dot(x, P8.spmv(y)), rel=1e-12)
    assert np.all(P8.spmv(x)[fixed] == 0)


def test_pcg_converges_and_reports_iterations(P8):
    R = P8.assemble(np.zeros(P8.neq), 0.1)
    x, k = P8.pcg(R, rtol=1e-10)
    assert k > 0
    r = R - P8.spmv(x)
    assert np.linalg.norm(r) <= 1e-9 * np.linalg.norm(R)
    x1, k1 = P8.pcg(R, rtol=1e-10, max_it=1)
    assert k1 == -1                                   # max_it reached


def test_zero_rhs_gives_zero_iterations(P8):
    P8.assemble(np.zeros(P8.neq), 0.1)
    x, k = P8.pcg(np.zeros(P8.neq))
    assert k == 0 and not x.any()


def test_newton_single_element_and_plasticity_onset():
    """edge case: a 1x1 mesh (one element, one colour) solves; a 40x40 mesh
    develops plastic points near the well by the last load step"""
    P1 = po.OracleProblem(po.default_params(1), nthreads=1)
    u = np.zeros(P1.neq)
    st, _ = P1.solve_steps(u, 2)
    assert st.converged and P1.n_colors == 1


def test_nan_input_propagates_to_residual(P8):
    u = np.zeros(P8.neq)
    u[10] = np.nan
    r = P8.assemble_residual(u, 0.1)
    assert np.isnan(r).any()


def test_learned_factor_gradient_matches_finite_differences():
    """the oracle's loss of the learned preconditioner (log Kaporin number of
    the triangular factor plus the (residual, increment) pair term,
    oracle/orc_mlp.py) against central differences of its gradient, on the
    oracle's own tangent of a 3 x 3 mesh; M is symmetric positive definite"""
    import scipy.sparse as sp
    from oracle import orc_mlp
    n = 3
    P = po.OracleProblem(po.default_params(n), nthreads=0)
    P.assemble(np.zeros(P.neq), 0.5)
    rp, col, K = P.arr("row_ptr").copy(), P.arr("col").copy(), P.arr("K").reshape(-1, 2, 2).copy()
    nn = P.n_nodes
    fixed = P.arr("fixed").astype(bool)
    A = sp.bsr_matrix((K, col, rp), shape=(2 * nn, 2 * nn)).tocsr()
    keep = sp.diags((~fixed).astype(float))
    A = (keep @ A @ keep).tocsr()
    dinv = np.where(fixed, 0.0, 1.0 / A.diagonal().clip(min=1e-300))
    rows = np.repeat(np.arange(nn), np.diff(rp))
    lut = {(int(rows[t]), int(col[t])): t for t in range(len(col))}

    def blocks(j, l):
        t = lut.get((int(j), int(l)))
        return K[t] if t is not None else np.zeros((2, 2))

    rng = np.random.default_rng(0)
    R = [rng.normal(size=P.neq) * ~fixed for _ in range(2)]
    E = [rng.normal(size=P.neq) * ~fixed for _ in range(2)]
    gr = 2 * n + 1
    O = rng.normal(size=(nn, 20)) * 0.1
    mv = lambda v: A @ v  # noqa: E731
    G = orc_mlp.factor(gr, gr, O, dinv)
    M = np.stack([orc_mlp.apply(gr, gr, G, dinv, np.eye(P.neq)[c]) for c in range(P.neq)], 1)
    assert np.abs(M - M.T).max() <= 1e-12 * np.abs(M).max()
    ev = np.linalg.eigvalsh(M[~fixed][:, ~fixed])
    assert ev.min() > 0
    loss, dO = orc_mlp.loss_grad_O(O, mv, blocks, gr, gr, dinv, R, E)
    for t in rng.choice(O.size, size=30, replace=False):
        h = 1e-6
        Op, Om = O.copy(), O.copy()
        Op.flat[t] += h
        Om.flat[t] -= h
        fd = (orc_mlp.loss_grad_O(Op, mv, blocks, gr, gr, dinv, R, E)[0] -
              orc_mlp.loss_grad_O(Om, mv, blocks, gr, gr, dinv, R, E)[0]) / (2 * h)
        assert abs(fd - dO.flat[t]) <= 1e-6 * max(1.0, abs(dO).max()), (t, fd, dO.flat[t])


def test_modified_thomas_newton_converges_in_fewer_iterations():
    """oracle: the accelerated load-stepped solve (main.cpp:194-217) reaches
    the same Newton tolerance in fewer iterations than the plain one, and both
    end at the same displacement to that tolerance"""
    out = {}
    for accel in (0, 1):
        P = po.OracleProblem(po.default_params(12), nthreads=0)
        u = np.zeros(P.neq)
        st, _ = P.solve_steps(u, 10, newton_max_it=40, accel=accel)
        assert st.converged
        out[accel] = (st.newton_iters, u)
    assert out[1][0] < out[0][0]
    assert np.abs(out[1][1] - out[0][1]).max() <= 1e-6 * np.abs(out[0][1]).max()


def test_block_jacobi_preconditioner():
    """the nodal block inverses invert the free part of every diagonal block,
    and block-Jacobi CG reaches the Jacobi-CG solution in fewer iterations"""
    P = po.OracleProblem(po.default_params(20), nthreads=4)
    u = np.zeros(P.neq)
    P.solve_steps(u, 10, step_begin=0, step_end=5, newton_max_it=30)
    R = P.assemble(u, 0.6)
    rp, col = P.arr("row_ptr"), P.arr("col")
    K, bi = P.arr("K").reshape(-1, 2, 2), P.arr("binv").reshape(-1, 2, 2)
    rows = np.repeat(np.arange(P.n_nodes), np.diff(rp))
    diag = K[rows == col]
    fx = P.arr("fixed").reshape(-1, 2).astype(bool)
    free = ~fx.any(1)
    assert np.abs(np.einsum("nij,njk->nik", bi[free], diag[free]) - np.eye(2)).max() < 1e-13
    one = fx[:, 0] & ~fx[:, 1]
    assert np.allclose(bi[one, 1, 1] * diag[one, 1, 1], 1.0) and not bi[one, 0].any() and not bi[one, :, 0].any()
    x0, k0 = P.pcg(R)
    P.set_block_jacobi(True)
    x1, k1 = P.pcg(R)
    assert 0 < k1 < 0.85 * k0, (k1, k0)
    assert np.abs(x1 - x0).max() < 1e-6 * np.abs(x0).max()


def test_resumable_newton_equals_solve_steps():
    """OracleNewton (the reference arm's timed Newton iterations) cut into
    chunks of 3 iterations gives the iterates, counts and committed state of
    orc_solve_steps bit for bit"""
    n, steps = 10, 6
    P1 = po.OracleProblem(po.default_params(n), nthreads=2)
    P2 = po.OracleProblem(po.default_params(n), nthreads=2)
    for P in (P1, P2):
        P.set_block_jacobi(True)
    u1, u2 = np.zeros(P1.neq), np.zeros(P2.neq)
    st, _ = P1.solve_steps(u1, steps, newton_max_it=40)
    N = po.OracleNewton(P2, steps, newton_max_it=40)
    its = cgs = 0
    while N.step < steps:
        d, c = N.advance(u2, 3)
        its += d
        cgs += c
    assert its == st.newton_iters and cgs == st.cg_iters
    assert np.array_equal(u1, u2)
    for f in ("eps_p", "sigma", "mtype", "alpha"):
        assert np.array_equal(P1.arr(f), P2.arr(f)), f


def _plastic_tangent_fd_error(consistent):
    """|K v - FD(v)| / |FD(v)| at the first Newton iterate of the last load
    step of a 20 x 20 ten-step solve, where points have gone plastic"""
    ctx = po.consistent_tangent() if consistent else contextlib.nullcontext()
    with ctx:
        P = po.OracleProblem(po.default_params(20), nthreads=2)
        u = np.zeros(P.neq)
        nw = po.OracleNewton(P, 10, newton_max_it=40, cg_rtol=1e-10)
        while not (nw.step == 9 and nw.open and nw.it >= 1):
            nw.advance(u, 1)
        lam = nw._lam()
        P.assemble(u, lam)
        rng = np.random.default_rng(1)
        v = rng.normal(size=P.neq)
        v[P.arr("fixed").astype(bool)] = 0
        Kv = P.spmv(v)
        h = 1e-6 * np.abs(u).max() / np.abs(v).max()
        fd = -(P.assemble_residual(u + h * v, lam) - P.assemble_residual(u - h * v, lam)) / (2 * h)
        return np.linalg.norm(Kv - fd) / np.linalg.norm(fd)


def test_consistent_tangent_matches_finite_differences_in_plastic_state():
    """The consistent variant of the oracle's tangent (spin factors from the
    projected principal stresses) is the derivative of the residual in a
    plastic state; the reference's TangentOperator is not, and the default
    switch gives the reference's tangent back."""
    e_ref = _plastic_tangent_fd_error(False)
    e_con = _plastic_tangent_fd_error(True)
    print("tangent vs finite differences: reference %.2e, consistent %.2e" % (e_ref, e_con))
    assert e_con < 5e-5 and e_ref > 1e-4
    assert _plastic_tangent_fd_error(False) == e_ref
