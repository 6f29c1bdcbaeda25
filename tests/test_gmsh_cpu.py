"""Gmsh meshes on the host: the reader (the reference reads its geometry with
TPZGmshReader, main.cpp:447-464), the generator of the reference's wellbore
meshes (gmsh/wellbore.geo), the order-2 problem with the reference's boundary
conditions (main.cpp:397-446, 546-601), and the oracle replaying the
reference's logged Newton runs on the reference's own mesh."""
import os

import numpy as np
import pytest

ip = pytest.importorskip("intpointsfem_gb300")
from intpointsfem_gb300 import gmsh_wellbore as gw  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

import replay_helpers as rh  # noqa: E402

from oracle.build import reference_dir  # noqa: E402

REF_GMSH = os.path.join(reference_dir(), "gmsh")


def _mesh(tmp_path, k):
    n, q = gw.REFERENCE_MESHES[k]
    path = str(tmp_path / ("wellbore_%d.msh" % k))
    gw.write_wellbore_msh(path, n, q)
    return ip.GmshMesh(path)


def _problem(g, cohesion=5.0, order=2):
    bcs, mat = gw.reference_bcs(cohesion)
    return ip.GmshProblem(g, bcs, order=order, **mat)


@pytest.mark.parametrize("k", [1, 2, 3])
def test_equation_and_colour_counts_match_the_logs(tmp_path, k):
    """equations and greedy colours of meshes 1-3 at orders 1, 2 and 3 equal
    the reference's logged "DOF" and "Number of colors" for them"""
    g = _mesh(tmp_path, k)
    n = gw.REFERENCE_MESHES[k][0]
    assert len(g.quads) == 4 * (n - 1) ** 2 and len(g.lines) == 8 * (n - 1) and len(g.points) == 4
    for order in (1, 2, 3):
        pb = _problem(g, order=order)
        run = rh.reference_run("CPU_NOT_MODIFIED/order%d-mesh%d" % (order, k))
        nc, _ = ip.color_elements(pb.array("connects"), pb.n_nodes, (order + 1) ** 2)
        assert pb.neq == run["dof"], (order, pb.neq, run["dof"])
        assert nc == run["colors"] == 4


@pytest.mark.parametrize("order", [1, 2, 3])
def test_element_geometry(tmp_path, order):
    """shape-function derivatives of every element sum to zero, a linear
    displacement field gives its constant strain at every point, the
    quadrature weights add up to the area of the polygonal annulus, and edge
    connects of neighbouring elements coincide"""
    g = _mesh(tmp_path, 1)
    pb = _problem(g, order=order)
    nn = (order + 1) ** 2
    dphi = pb.array("dphi").reshape(-1, nn, 2, nn)
    con = pb.array("connects").reshape(-1, nn)
    xy = pb.array("node_xy").reshape(-1, 2)
    assert np.abs(dphi.sum(-1)).max() < 1e-11
    ux, uy = 1e-3 * xy[:, 0] + 2e-3 * xy[:, 1], -0.5e-3 * xy[:, 0] + 3e-3 * xy[:, 1]
    exx = np.einsum("eqn,en->eq", dphi[:, :, 0, :], ux[con])
    gxy = np.einsum("eqn,en->eq", dphi[:, :, 1, :], ux[con]) + np.einsum("eqn,en->eq", dphi[:, :, 0, :], uy[con])
    eyy = np.einsum("eqn,en->eq", dphi[:, :, 1, :], uy[con])
    assert np.abs(exx - 1e-3).max() < 1e-12 and np.abs(gxy - 1.5e-3).max() < 1e-12
    assert np.abs(eyy - 3e-3).max() < 1e-12
    r, th = gw.wellbore_nodes(*gw.REFERENCE_MESHES[1])
    area = 0.5 * len(th) * np.sin(2 * np.pi / len(th)) * (r[-1] ** 2 - r[0] ** 2)
    assert abs(pb.array("weight").sum() - area) < 1e-10 * area
    # every connect is used, and no two connects share a position
    assert np.unique(con).size == pb.n_nodes
    assert np.unique(np.round(xy, 12), axis=0).shape[0] == pb.n_nodes


@pytest.mark.skipif(not os.path.isdir(REF_GMSH), reason="reference meshes not present")
@pytest.mark.parametrize("k", [1, 2])
def test_generator_reproduces_the_reference_meshes(tmp_path, k):
    """same quadrilaterals, boundary lines, tagged points and physical names as
    gmsh/wellbore_k.msh; coordinates within Gmsh's progression round-off"""
    a = _mesh(tmp_path, k)
    b = ip.GmshMesh(os.path.join(REF_GMSH, "wellbore_%d.msh" % k))
    assert a.physical == b.physical
    assert a.xy.shape == b.xy.shape
    spatial = pytest.importorskip("scipy.spatial")
    dist, idx = spatial.cKDTree(a.xy).query(b.xy)
    assert dist.max() < 1e-7
    assert set(map(tuple, np.sort(a.quads, 1))) == set(map(tuple, np.sort(idx[b.quads], 1)))
    assert set(map(tuple, np.sort(a.lines, 1))) == set(map(tuple, np.sort(idx[b.lines], 1)))
    assert set(zip(a.points.tolist(), a.point_phys.tolist())) == set(zip(idx[b.points].tolist(),
                                                                          b.point_phys.tolist()))


def test_boundary_loads_and_constraints(tmp_path):
    """normal stress v on the well: zero net force, and sum f.x = v * (-2 A)
    for the polygonal hole of area A (divergence theorem); fixed_x / fixed_y
    fix one component at two points each"""
    g = _mesh(tmp_path, 1)
    v = -10.0
    pb = ip.GmshProblem(g, [("bc_wellbore", 6, v), ("fixed_x", 3, 1, 0), ("fixed_y", 3, 0, 1)], 2000.0, 0.2, 5.0,
                        20.0)
    f = pb.array("df").reshape(-1, 2)
    xy = pb.array("node_xy").reshape(-1, 2)
    assert abs(f[:, 0].sum()) < 1e-12 and abs(f[:, 1].sum()) < 1e-12
    th = gw.wellbore_nodes(*gw.REFERENCE_MESHES[1])[1]
    area = 0.5 * len(th) * 0.1 ** 2 * np.sin(2 * np.pi / len(th))
    assert abs((f * xy).sum() - v * (-2.0 * area)) < 1e-12
    fixed = pb.array("fixed").reshape(-1, 2)
    assert fixed.sum() == 4
    for comp, pts in ((0, [(0.0, 4.0), (0.0, -4.0)]), (1, [(4.0, 0.0), (-4.0, 0.0)])):
        for p in pts:
            node = np.argmin(((xy - p) ** 2).sum(1))
            assert fixed[node, comp] == 1 and fixed[node, 1 - comp] == 0


def test_reader_and_problem_reject_what_they_do_not_support(tmp_path):
    good = tmp_path / "good.msh"
    gw.write_wellbore_msh(str(good), 4, 1.2)
    txt = good.read_text()
    cases = {
        "ver.msh": txt.replace("4.1 0 8", "2.2 0 8"),
        "bin.msh": txt.replace("4.1 0 8", "4.1 1 8"),
        "tri.msh": txt.replace("2 1 3 9", "2 1 2 9", 1),
        "z.msh": txt.replace("\n0.10000000000000001 0 0\n", "\n0.10000000000000001 0 1\n", 1),
    }
    for name, body in cases.items():
        p = tmp_path / name
        p.write_text(body)
        with pytest.raises(ip.IpfemError):
            ip.GmshMesh(str(p))
    with pytest.raises(ip.IpfemError):
        ip.GmshMesh(str(tmp_path / "missing.msh"))
    g = ip.GmshMesh(str(good))
    with pytest.raises(ip.IpfemError):
        ip.GmshProblem(g, [(99, 6, -1.0)], 2000.0, 0.2, 5.0, 20.0)         # no entity with that tag
    with pytest.raises(ip.IpfemError):
        ip.GmshProblem(g, [("fixed_x", 6, -1.0)], 2000.0, 0.2, 5.0, 20.0)  # traction on points
    with pytest.raises(ip.IpfemError):
        ip.GmshProblem(g, [("bc_wellbore", 0, 1.0)], 2000.0, 0.2, 5.0, 20.0)  # non-zero Dirichlet
    with pytest.raises(ip.IpfemError):
        ip.GmshProblem(g, [("bc_wellbore", 2, 1.0)], 2000.0, 0.2, 5.0, 20.0)  # unsupported type


def _oracle(pb, cohesion=5.0):
    prm = po.default_params(4, E=2000.0, nu=0.2, cohesion=cohesion, phi_deg=20.0, psi_deg=20.0, sxx0=0.0,
                            syy0=0.0, szz0=0.0, sxy0=0.0)
    mesh = {k: pb.array(k) for k in ("node_xy", "connects", "fixed", "f0", "df")}
    mesh["order"] = pb.order
    return po.OracleProblem(prm, mesh=mesh)


@pytest.mark.parametrize("order", [1, 3])
def test_oracle_element_blocks_equal_the_library_blocks(tmp_path, order):
    """the oracle's own element blocks (recomputed from the coordinates) hold
    the library's dphi and weights bit for bit"""
    pb = _problem(_mesh(tmp_path, 1), order=order)
    P = _oracle(pb)
    nn = nq = (order + 1) ** 2
    nd = 2 * nn
    B = P.arr("B").reshape(-1, nq, 3, nd)
    d = pb.array("dphi").reshape(-1, nq, 2, nn)
    assert np.array_equal(B[:, :, 0, 0::2], d[:, :, 0, :]) and np.array_equal(B[:, :, 1, 0::2], d[:, :, 1, :])
    assert np.array_equal(B[:, :, 1, 1::2], d[:, :, 0, :]) and np.array_equal(B[:, :, 2, 1::2], d[:, :, 1, :])
    assert np.array_equal(P.arr("weight"), pb.array("weight"))


def test_oracle_replays_the_order_1_logs(tmp_path):
    """order 1 (NeoPZ's order-1 basis is the bilinear Lagrange basis, so the
    residual norms themselves are comparable): initial stiffness on mesh 1,
    ratios within 0.003 of the logged ones (limit 0.5282 to 1e-4) and norms
    within 1 %; modified Thomas within 0.01 per ratio"""
    pb = _problem(_mesh(tmp_path, 1), order=1)
    for accel, variant in ((0, "CPU_NOT_MODIFIED"), (1, "CPU_MODIFIED")):
        P = _oracle(pb)
        ref = rh.reference_run(variant + "/order1-mesh1")
        n_run = len(ref["residue"])
        st, log = P.solve_steps(np.zeros(P.neq), 1, newton_rtol=1e-14, newton_max_it=n_run, cg_rtol=1e-11,
                                tangent_mode=1, accel=accel)
        ours, refr = log[:, 2], np.asarray(ref["residue"])
        diff = np.abs(rh.ratios(ours) - rh.ratios(refr)).max()
        print("order 1 %s: max ratio difference %.4f, first norms %.6f / %.6f" % (variant, diff, ours[0], refr[0]))
        if accel == 0:
            assert diff < 0.003 and abs(rh.ratios(ours)[-1] - rh.ratios(refr)[-1]) < 1e-4
            assert np.abs(ours / refr - 1).max() < 0.01
        else:
            assert diff < 0.01


@pytest.mark.parametrize("accel,variant,iters,tol_early,tol_late", [
    (0, "CPU_NOT_MODIFIED", 12, 0.03, 0.006),
    (1, "CPU_MODIFIED", 7, 0.01, 0.02),
])
def test_oracle_replays_the_logged_runs(tmp_path, accel, variant, iters, tol_early, tol_late):
    """The oracle, on mesh 1 with the verification configuration, runs the
    initial-stiffness iteration (plain and modified-Thomas) that produced the
    reference's logs; the successive residual ratios agree with the logged
    ones (0.5426 in the limit of the plain iteration) and the reference's
    total residual reduction takes the same number of iterations."""
    pb = _problem(_mesh(tmp_path, 1))
    P = _oracle(pb)
    u = np.zeros(P.neq)
    ref = rh.reference_run(variant + "/order2-mesh1")
    n_run = iters if accel == 0 else ref["iterations"]
    st, log = P.solve_steps(u, 1, newton_rtol=1e-14, newton_max_it=n_run, cg_rtol=1e-11, tangent_mode=1, accel=accel)
    ours = log[:, 2]
    assert len(ours) == n_run
    early, late, it_ours, it_ref = rh.compare(ours, ref["residue"][:n_run], n_run - 1)
    print("%s: ratio differences %.4f / %.4f" % (variant, early, late))
    assert early < tol_early and late < tol_late
    if accel == 0:
        assert abs(rh.ratios(ours)[-1] - rh.ratios(ref["residue"])[-1]) < 1e-3
    else:
        assert it_ours == it_ref == ref["iterations"]


@pytest.mark.parametrize("order", [1, 2, 3])
def test_mixed_mesh_triangles(tmp_path, order):
    """triangles (two quadrants split, as wellbore.geo leaves the surfaces it
    does not recombine) of order p in the order-p block shape: ghost columns
    zero and ghost dofs fixed, Lagrange connects shared with the neighbouring
    quadrilaterals, a linear field's strain exact, the quadrature area equal to
    the all-quadrilateral mesh's, and the equations without ghosts as counted
    from the mesh's vertices, edges and faces"""
    path = str(tmp_path / "mix.msh")
    gw.write_wellbore_msh(path, 9, 1.3, tri_quadrants=(1, 3))
    g = ip.GmshMesh(path)
    assert len(g.tris) == 2 * 2 * 8 * 8 and len(g.quads) == 2 * 8 * 8
    pb = _problem(g, order=order)
    nn, nt = (order + 1) ** 2, (order + 1) * (order + 2) // 2
    shape = pb.array("el_shape").astype(bool)
    assert shape.sum() == len(g.tris)
    dphi = pb.array("dphi").reshape(-1, nn, 2, nn)
    con = pb.array("connects").reshape(-1, nn)
    xy = pb.array("node_xy").reshape(-1, 2)
    fixed = pb.array("fixed").reshape(-1, 2)
    assert not dphi[shape][:, :, :, nt:].any()
    ghosts = np.unique(con[shape][:, nt:])
    assert ghosts.size == pb.n_ghost == shape.sum() * (nn - nt) and fixed[ghosts].all()
    ux = 1e-3 * xy[:, 0] + 2e-3 * xy[:, 1]
    assert np.abs(np.einsum("eqn,en->eq", dphi[:, :, 0, :], ux[con]) - 1e-3).max() < 1e-12
    assert np.abs(np.einsum("eqn,en->eq", dphi[:, :, 1, :], ux[con]) - 2e-3).max() < 1e-12
    gw.write_wellbore_msh(str(tmp_path / "q.msh"), 9, 1.3)
    area_q = _problem(ip.GmshMesh(str(tmp_path / "q.msh")), order=order).array("weight").sum()
    assert abs(pb.array("weight").sum() - area_q) < 1e-12 * area_q
    V = len(g.xy)
    E = (4 * len(g.quads) + 3 * len(g.tris) + 8 * 8) // 2
    real = V + (order - 1) * E + (order - 1) ** 2 * len(g.quads) + (1 if order == 3 else 0) * len(g.tris)
    assert pb.n_equations == 2 * real
    nc, _ = ip.color_elements(con, pb.n_nodes, nn)
    assert nc <= 16


@pytest.mark.skipif(not os.path.isdir(REF_GMSH), reason="reference meshes not present")
def test_reference_mixed_mesh_reads(tmp_path):
    g = ip.GmshMesh(os.path.join(REF_GMSH, "wellbore_mix.msh"))
    assert len(g.quads) == 64 and len(g.tris) == 208 and len(g.lines) == 48 and len(g.points) == 4
    for order in (1, 2, 3):
        pb = _problem(g, order=order)
        assert pb.n_el == 272 and pb.array("el_shape").sum() == 208
