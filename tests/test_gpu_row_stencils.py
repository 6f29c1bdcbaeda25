"""Row stencils of the SpMVs (ipfem_set_row_stencils): on the structured
wellbore grid every row's block columns come from a few dozen offset
patterns; the SpMVs that read them must give the same bits as the ones that
read the stored column indices, in every solver that uses them (plain FP64
CG, FP32 CG, flexible CG with the learned factor, the training pass).  The
plain FP64 path with stencils (the default) is also compared with the oracle
bit for bit by test_gpu_parity.py."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ip = pytest.importorskip("intpointsfem_gb300")
torch = pytest.importorskip("torch")


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.int64)


def _matrix(n, **kw):
    return ip.ElastoPlasticIntPointsStructMatrix(ip.WellboreMesh(ip.wellbore_params(n, **kw)))


def test_stencil_counts():
    sm = _matrix(12)
    n64, n32 = sm.row_stencil_count()
    assert 0 < n64 <= 255 and n32 == 0
    sm.set_precision(ip.MIXED)
    n64b, n32 = sm.row_stencil_count()
    assert n64b == n64 and 0 < n32 <= 255
    print("row stencils at 12 x 12: FP64 layout %d, FP32 layout %d" % (n64, n32))


def test_layout_info():
    """the FP64 layout holds every block; the FP32 one holds the diagonal and
    the upper blocks while the stencils are on, and every block without them"""
    sm = _matrix(12)
    nb, nn = sm.n_blocks, sm.n_nodes
    stored, slots, upper = sm.layout_info()
    assert (stored, upper) == (nb, False) and slots >= nb
    with pytest.raises(ip.IpfemError):
        sm.layout_info(fp32=True)
    sm.set_precision(ip.MIXED)
    stored, slots, upper = sm.layout_info(fp32=True)
    assert upper and stored == (nb + nn) // 2 and stored <= slots < nb
    sm.set_row_stencils(0)
    stored, slots, upper = sm.layout_info(fp32=True)
    assert (stored, upper) == (nb, False) and slots >= nb


def test_order3_rows_keep_explicit_columns(tmp_path):
    """order-3 vertex rows have 49 blocks: longer than a stencil, so the
    layout keeps its column indices and the solve is unchanged"""
    from intpointsfem_gb300 import gmsh_wellbore as gw
    path = str(tmp_path / "w.msh")
    gw.write_wellbore_msh(path, 6, 1.175)
    bcs, mat = gw.reference_bcs()
    pb = ip.GmshProblem(ip.GmshMesh(path), bcs, order=3, **mat)
    sm = ip.ElastoPlasticIntPointsStructMatrix(pb)
    assert sm.row_stencil_count() == (0, 0)


@pytest.mark.parametrize("prec", [ip.PREC_JACOBI, ip.PREC_BLOCK_JACOBI])
def test_plain_newton_same_bits(prec):
    out = []
    for on in (1, 0):
        sm = _matrix(40)
        sm.set_row_stencils(on)
        sm.set_preconditioner(prec)
        u = np.zeros(sm.neq)
        st, log = sm.newton(u, 10, newton_max_it=30)
        assert st.converged
        out.append((u, st.cg_iters, log))
    (ua, ka, la), (ub, kb, lb) = out
    assert ka == kb and np.array_equal(_bits(ua), _bits(ub)) and np.array_equal(_bits(la), _bits(lb))


def test_toggle_inside_one_context():
    """switching the mode drops the captured CG graphs: the same context
    solves with both SpMVs and gets the same bits"""
    sm = _matrix(16)
    sm.SetLoadFactor(0.8)
    b = sm.assemble(np.zeros(sm.neq), np.zeros(sm.neq))
    xa, ia = sm.solve(b, rtol=1e-9)
    sm.set_row_stencils(0)
    xb, ib = sm.solve(b, rtol=1e-9)
    sm.set_row_stencils(1)
    xc, ic = sm.solve(b, rtol=1e-9)
    assert ia == ib == ic > 0
    assert np.array_equal(_bits(xa), _bits(xb)) and np.array_equal(_bits(xa), _bits(xc))


@pytest.mark.parametrize("learned", [False, True])
def test_mixed_newton_same_bits(learned):
    from intpointsfem_gb300 import train_preconditioner as tp
    n = 40
    out = []
    for on in (1, 0):
        sm = _matrix(n)
        sm.set_row_stencils(on)
        sm.set_precision(ip.MIXED)
        if learned:
            sm.set_node_grid(2 * n + 1, 2 * n + 1)
            sm.mlp_init(0)
            sm.set_mlp_params(tp.load_weights())
            sm.set_preconditioner(ip.PREC_MLP)
        u = np.zeros(sm.neq)
        st, _ = sm.newton(u, 10, newton_max_it=40, cg_rtol=1e-4)
        assert st.converged
        out.append((u, st.cg_iters))
    (ua, ka), (ub, kb) = out
    assert ka == kb and np.array_equal(_bits(ua), _bits(ub))


def test_learn_grad_same_bits():
    from intpointsfem_gb300 import learned
    wb, sm = learned.make_solver(24, -15.0, 30.0, seed=3)
    u = torch.zeros(sm.neq, dtype=torch.float64, device="cuda")
    sm.SetLoadFactor(0.6)
    sm.assemble(u, torch.zeros_like(u), ip.DEVICE)
    g = torch.Generator(device="cuda").manual_seed(1)
    r = torch.randn(3, sm.neq, device="cuda", generator=g)
    e = torch.randn(3, sm.neq, device="cuda", generator=g)
    ga, la = sm.learn_grad(r, e, 3, 1.0, 1.0)
    # without stencils the FP32 tangent lives in the full layout: assembled again
    sm.set_row_stencils(0)
    sm.assemble(u, torch.zeros_like(u), ip.DEVICE)
    gb, lb = sm.learn_grad(r, e, 3, 1.0, 1.0)
    assert la == lb and np.array_equal(ga.view(np.int32), gb.view(np.int32))
