"""The FP32 residual kernels (ipfem_gather_strain32, ipfem_scatter_residual32)
against an exact host emulation of their arithmetic, at element orders 1, 2
and 3, with a partial last tile of 32 elements:
  - strain: each displacement taken relative to its element's first connect
    (same component) in FP64 and rounded to FP32, then the FP32 fma chains
    exx = sum dNx ux, gxy = sum (dNy ux, dNx uy), eyy = sum dNy uy in node order;
  - element forces: per node and component, the FP32 fma chain over the points
    (dNx sxx, dNy sxy | dNx sxy, dNy syy), negated; the colour slabs summed in
    FP32 in the reference's pairwise slab order (TPZNumericalIntegrator.cpp:69-77)
    and widened to FP64.
The emulated fma (fp32_emul.fma32) is correctly rounded; test_fp32_emul_cpu.py
checks it."""
import numpy as np
import pytest

from fp32_emul import fma32

pytestmark = pytest.mark.gpu

ip = pytest.importorskip("intpointsfem_gb300")
torch = pytest.importorskip("torch")


def _problems():
    from intpointsfem_gb300 import gmsh_wellbore as gw
    yield "wellbore order 2", lambda tmp: ip.WellboreMesh(ip.wellbore_params(10))
    for order in (1, 3):
        def make(tmp, order=order):
            path = str(tmp / ("w%d.msh" % order))
            gw.write_wellbore_msh(path, 6, 1.175)
            bcs, mat = gw.reference_bcs()
            return ip.GmshProblem(ip.GmshMesh(path), bcs, order=order, **mat)
        yield "gmsh order %d" % order, make


@pytest.mark.parametrize("name,make", list(_problems()), ids=[p[0] for p in _problems()])
def test_fp32_kernels_equal_exact_emulation(tmp_path, name, make):
    pb = make(tmp_path)
    sm = ip.ElastoPlasticIntPointsStructMatrix(pb)
    sm.set_precision(ip.MIXED)
    sm.set_residual_precision(32)
    n_el, n_ip = sm.n_el, sm.n_ip
    nq = n_ip // n_el
    nn = nq
    assert n_el % 32 != 0, "the last tile should be partial"
    dphi = sm.get_setup(3).reshape(n_el, nq, 2, nn).astype(np.float32)
    dofs = sm.get_setup(2).reshape(n_el, 2 * nn)
    colour = sm.get_setup(0)
    n_colors = int(sm.get_setup(1)[0])
    rng = np.random.default_rng(11)
    xy = pb.array("node_xy").reshape(-1, 2)
    # a smooth far field plus a small local variation, as in a load step
    u = np.empty(sm.neq)
    u[0::2] = 1e-2 * xy[:, 0] + 1e-5 * rng.normal(size=sm.n_nodes)
    u[1::2] = -7e-3 * xy[:, 1] + 1e-5 * rng.normal(size=sm.n_nodes)

    # strain
    du = torch.tensor(u, device="cuda")
    ds = torch.zeros(3 * n_ip, dtype=torch.float32, device="cuda")
    sm.gather_strain32(du, ds)
    ue = (u[dofs] - u[dofs[:, [0, 1] * nn]]).astype(np.float32)     # [n_el, 2nn]
    ux, uy = ue[:, 0::2], ue[:, 1::2]
    dx, dy = dphi[:, :, 0, :], dphi[:, :, 1, :]                     # [n_el, nq, nn]
    exx = np.zeros((n_el, nq), np.float32)
    gxy = np.zeros_like(exx)
    eyy = np.zeros_like(exx)
    for n in range(nn):
        exx = fma32(dx[:, :, n], ux[:, None, n], exx)
    for n in range(nn):
        gxy = fma32(dy[:, :, n], ux[:, None, n], gxy)
        gxy = fma32(dx[:, :, n], uy[:, None, n], gxy)
    for n in range(nn):
        eyy = fma32(dy[:, :, n], uy[:, None, n], eyy)
    want = np.stack([exx.ravel(), gxy.ravel(), eyy.ravel()])
    got = ds.cpu().numpy().reshape(3, n_ip)
    assert np.array_equal(got.view(np.int32), want.view(np.int32))

    # element forces and colour sums
    sig = (rng.normal(size=(3, n_ip)) * 10.0).astype(np.float32)
    dsig = torch.tensor(sig.ravel(), device="cuda")
    dres = torch.zeros(sm.neq, dtype=torch.float64, device="cuda")
    sm.scatter_residual32(dsig, dres)
    sxx, sxy, syy = (sig[k].reshape(n_el, nq) for k in range(3))
    fx = np.zeros((n_el, nn), np.float32)
    fy = np.zeros_like(fx)
    for q in range(nq):
        nx, ny = dx[:, q, :], dy[:, q, :]
        fx = fma32(nx, sxx[:, q, None], fx)
        fx = fma32(ny, sxy[:, q, None], fx)
        fy = fma32(nx, sxy[:, q, None], fy)
        fy = fma32(ny, syy[:, q, None], fy)
    fe = np.empty((n_el, 2 * nn), np.float32)
    fe[:, 0::2], fe[:, 1::2] = -fx, -fy
    slabs = np.zeros((n_colors, sm.neq), np.float32)
    for c in range(n_colors):
        els = np.nonzero(colour == c)[0]
        slabs[c, dofs[els].ravel()] = fe[els].ravel()     # one element of a colour per node
    nc, ca = n_colors, n_colors // 2
    while ca > 0:
        first = nc - ca
        for k in range(ca):
            slabs[k] = slabs[k] + slabs[first + k]
        nc -= ca
        ca = nc // 2
    want_res = slabs[0].astype(np.float64)
    assert np.array_equal(dres.cpu().numpy(), want_res)
