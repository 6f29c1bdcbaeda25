"""Gmsh meshes on the GPU: the order-2 problem on the reference's own
wellbore meshes (generated here from gmsh/wellbore.geo's recipe, identical to
the shipped files up to Gmsh's progression round-off).
  - bit-exact against the oracle on an unstructured-numbered mesh, for the
    full-tangent, initial-stiffness and modified-Thomas iterations;
  - the reference's logged runs replayed on meshes 1 and 2: the successive
    residual ratios of the initial-stiffness iteration agree with the logged
    ones (the limit to 1e-3: 0.5426 on mesh 1, 0.5385 on mesh 2) and the
    reference's total residual reduction takes the same number of iterations
    (+-1); the modified-Thomas runs agree to 0.03 in every ratio and +-1
    iteration (their acceleration factor depends on the basis)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ip = pytest.importorskip("intpointsfem_gb300")
from intpointsfem_gb300 import gmsh_wellbore as gw  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

import replay_helpers as rh  # noqa: E402


def _problem(tmp_path, n, q, cohesion=5.0, order=2):
    path = str(tmp_path / ("wb_%d.msh" % n))
    gw.write_wellbore_msh(path, n, q)
    bcs, mat = gw.reference_bcs(cohesion)
    return ip.GmshProblem(ip.GmshMesh(path), bcs, order=order, **mat)


def _oracle(pb, cohesion=5.0):
    prm = po.default_params(4, E=2000.0, nu=0.2, cohesion=cohesion, phi_deg=20.0, psi_deg=20.0, sxx0=0.0,
                            syy0=0.0, szz0=0.0, sxy0=0.0)
    mesh = {k: pb.array(k) for k in ("node_xy", "connects", "fixed", "f0", "df")}
    mesh["order"] = pb.order
    return po.OracleProblem(prm, mesh=mesh)


@pytest.mark.parametrize("order,tangent,accel", [(2, 0, 0), (2, 1, 0), (2, 1, 1), (1, 0, 0), (1, 1, 1), (3, 0, 0),
                                                 (3, 1, 1)])
def test_gmsh_problem_bit_exact_with_oracle(tmp_path, order, tangent, accel):
    pb = _problem(tmp_path, 9, 1.3, order=order)
    sm = ip.ElastoPlasticIntPointsStructMatrix(pb)
    P = _oracle(pb)
    assert sm.n_colors == P.n_colors == 4
    sm.set_newton_tangent(tangent)
    sm.set_newton_accel(accel)
    ug, uo = np.zeros(sm.neq), np.zeros(sm.neq)
    sg, lg = sm.newton(ug, 1, newton_rtol=1e-12, newton_max_it=6, cg_rtol=1e-10)
    so, lo = P.solve_steps(uo, 1, newton_rtol=1e-12, newton_max_it=6, cg_rtol=1e-10, tangent_mode=tangent,
                           accel=accel)
    assert sg.newton_iters == so.newton_iters and sg.cg_iters == so.cg_iters
    assert np.array_equal(lg, lo)
    assert np.array_equal(ug, uo)
    assert np.abs(ug).max() > 1e-4
    # the state committed at the accepted step
    n_ip = P.n_ip
    sg_state = sm.get_state(1).reshape(4, n_ip)
    so_state = P.arr("sigma").reshape(n_ip, 6)
    assert np.array_equal(sg_state[0], so_state[:, 0]) and np.array_equal(sg_state[2], so_state[:, 3])
    assert np.array_equal(sm.get_state(3), P.arr("mtype").astype(np.float64))


@pytest.mark.parametrize("k", [1, 2])
@pytest.mark.parametrize("accel", [0, 1])
def test_replay_of_the_logged_runs(tmp_path, k, accel):
    n, q = gw.REFERENCE_MESHES[k]
    pb = _problem(tmp_path, n, q)
    sm = ip.ElastoPlasticIntPointsStructMatrix(pb)
    sm.set_newton_tangent(1)
    sm.set_newton_accel(accel)
    variant = "CPU_MODIFIED" if accel else "CPU_NOT_MODIFIED"
    ref = rh.reference_run("%s/order2-mesh%d" % (variant, k))
    assert sm.neq == ref["dof"] and sm.n_colors == ref["colors"]
    # one iteration past the logged ones for the accelerated runs: their factor
    # alpha is a ratio of Euclidean dot products of coefficient vectors, which
    # depends on the basis, so their iterates differ slightly from NeoPZ's
    n_run = len(ref["residue"]) + 1 if accel else min(len(ref["residue"]), 24)
    u = np.zeros(sm.neq)
    st, log = sm.newton(u, 1, newton_rtol=1e-14, newton_max_it=n_run, cg_rtol=1e-11)
    ours = log[:, 2]
    early, late, it_ours, it_ref = rh.compare(ours, ref["residue"], len(ref["residue"]) - 1)
    print("mesh %d %s: %d equations, ratio differences %.4f (first 3) / %.4f (rest), iterations to the reference's "
          "reduction %s vs %s, last ratios %s vs %s"
          % (k, variant, sm.neq, early, late, it_ours, it_ref, np.round(rh.ratios(ours)[-3:], 4),
             np.round(rh.ratios(ref["residue"])[-3:], 4)))
    print("  ratios ours %s\n  ratios ref  %s" % (np.round(rh.ratios(ours)[:10], 4),
                                                    np.round(rh.ratios(ref["residue"])[:10], 4)))
    if accel == 0:
        assert early < 0.03 and late < 0.015
        assert abs(rh.ratios(ours)[-1] - rh.ratios(ref["residue"])[-1]) < 1e-3
        assert abs(it_ours - it_ref) <= 1
    else:
        assert early < 0.02 and late < 0.03
        assert it_ours is not None and abs(it_ours - it_ref) <= 1


@pytest.mark.parametrize("order,k", [(1, 1), (1, 2), (3, 1), (3, 2)])
def test_replay_of_the_logged_runs_orders_1_and_3(tmp_path, order, k):
    """orders 1 and 3 on meshes 1 and 2, initial stiffness: the whole logged
    run (order 3 converges slowly, 251 and 179 iterations, with the limit
    ratio 0.9632 / 0.9547) and its limit ratio to 2e-3; for order 1 (NeoPZ's
    order-1 basis is the bilinear Lagrange basis) also the ratio sequence, the
    norms themselves and the iteration count.  For order 3 the transient
    ratios depend on the basis (NeoPZ's hierarchical cubic functions against
    Lagrange ones), the limit does not.  Then the modified-Thomas run's
    iteration count to the logged reduction."""
    n, q = gw.REFERENCE_MESHES[k]
    pb = _problem(tmp_path, n, q, order=order)
    ref = rh.reference_run("CPU_NOT_MODIFIED/order%d-mesh%d" % (order, k))
    sm = ip.ElastoPlasticIntPointsStructMatrix(pb)
    assert sm.neq == ref["dof"] and sm.n_colors == ref["colors"]
    sm.set_newton_tangent(1)
    n_run = len(ref["residue"])
    st, log = sm.newton(np.zeros(sm.neq), 1, newton_rtol=1e-14, newton_max_it=n_run, cg_rtol=1e-11,
                        log_cap=n_run + 8)
    ours, refr = log[:, 2], np.asarray(ref["residue"])
    ro, rr = rh.ratios(ours), rh.ratios(refr)
    early, late, it_ours, it_ref = rh.compare(ours, refr, n_run - 1)
    print("order %d mesh %d: %d equations, ratio differences %.4f / %.4f, limit %.4f vs %.4f, iterations to the "
          "reference's reduction %s vs %s, first norms %.5g / %.5g"
          % (order, k, sm.neq, early, late, ro[-1], rr[-1], it_ours, it_ref, ours[0], refr[0]))
    assert abs(ro[-1] - rr[-1]) < 2e-3
    if order == 1:
        assert it_ours is not None and abs(it_ours - it_ref) <= 1
        assert late < 0.006 and np.abs(ours / refr - 1).max() < 0.02
    refm = rh.reference_run("CPU_MODIFIED/order%d-mesh%d" % (order, k))
    sm2 = ip.ElastoPlasticIntPointsStructMatrix(pb)
    sm2.set_newton_tangent(1)
    sm2.set_newton_accel(1)
    n_m = 2 * len(refm["residue"]) if order == 3 else len(refm["residue"]) + 4
    st2, log2 = sm2.newton(np.zeros(sm2.neq), 1, newton_rtol=1e-14, newton_max_it=n_m, cg_rtol=1e-11,
                           log_cap=n_m + 8)
    _, _, itm_ours, itm_ref = rh.compare(log2[:, 2], refm["residue"], len(refm["residue"]) - 1)
    print("  modified Thomas: iterations to the reference's reduction %s vs %s" % (itm_ours, itm_ref))
    assert itm_ours is not None
    if order == 1:
        assert abs(itm_ours - itm_ref) <= 1
    else:
        # the residual norms of the cubic bases weight the slow modes differently,
        # so only the scale of the count compares
        assert itm_ours <= 1.5 * itm_ref


@pytest.mark.parametrize("order", [1, 3])
def test_mixed_precision_orders_1_and_3(tmp_path, order):
    """the FP32 tangent and FP32 CG of the mixed solve at orders 1 and 3:
    the same Newton solution as plain FP64 to the Newton tolerance"""
    pb = _problem(tmp_path, 16, 1.3, order=order)
    u = {}
    for prec in (ip.PLAIN_FP64, ip.MIXED):
        sm = ip.ElastoPlasticIntPointsStructMatrix(pb)
        sm.set_precision(prec)
        uu = np.zeros(sm.neq)
        st, _ = sm.newton(uu, 1, newton_rtol=1e-10, newton_max_it=40,
                          cg_rtol=1e-4 if prec == ip.MIXED else 1e-10)
        assert st.converged
        u[prec] = uu
    err = np.abs(u[ip.MIXED] - u[ip.PLAIN_FP64]).max() / np.abs(u[ip.PLAIN_FP64]).max()
    assert err < 1e-7, err


def test_line_probe_of_the_solution_matches_the_reference_fem(tmp_path):
    """The reference's verification configuration on mesh 2 (order 2, the
    logged initial-stiffness iteration to convergence), post-processed like
    the reference's data: a 1001-point probe along y = 0 written with the
    columns of its CSVs.  Against its finite-element profile
    (ElastoPlasticFEMdata.csv, made on a coarser mesh that is not shipped:
    about 20 radial nodes with progression 1.25): radial displacement within
    2 % (measured 1.4 %), stresses beyond the first element layer within 5 %
    (3.1 %), and the plastic radius (FailureType) at the RK solution's 0.162
    (0.1624)."""
    from intpointsfem_gb300 import postprocess as pp
    import verification_helpers as vh

    n, q = gw.REFERENCE_MESHES[2]
    pb = _problem(tmp_path, n, q)
    sm = ip.ElastoPlasticIntPointsStructMatrix(pb)
    sm.set_newton_tangent(1)
    u = np.zeros(sm.neq)
    st, _ = sm.newton(u, 1, newton_rtol=1e-10, newton_max_it=80, cg_rtol=1e-11)
    assert st.converged
    S = pp.Solution.from_struct_matrix(pb, sm, u)
    rows = S.write_line_probe_csv(str(tmp_path / "probe.csv"), (0.1, 0.0), (4.0, 0.0), 1001)
    with open(tmp_path / "probe.csv") as f:
        assert [h.strip('"') for h in f.readline().strip().split(",")] == pp.COLUMNS
    c = {k: i for i, k in enumerate(pp.COLUMNS)}
    fem = vh.fixture()["ep_fem"]                   # x, u_x, s_xx, s_yy, s_zz, ep_xx, ep_yy
    x = rows[:, c["Points:0"]]
    assert rows[:, c["vtkValidPointMask"]].min() == 1.0
    eu = np.abs(rows[:, c["Displacement:0"]] - np.interp(x, fem[:, 0], fem[:, 1])).max() / np.abs(fem[:, 1]).max()
    beyond = x > 0.12
    sc = np.abs(fem[:, 2]).max()
    es = max(np.abs(rows[beyond, c[col]] - np.interp(x[beyond], fem[:, 0], fem[:, k])).max() / sc
             for col, k in (("Stress:0", 2), ("Stress:4", 3), ("Stress:8", 4)))
    plastic = x[rows[:, c["FailureType"]] > 0.5]
    print("line probe vs reference FEM: u %.2e, stresses %.2e, plastic to r = %.4f" % (eu, es, plastic.max()))
    assert eu < 2e-2 and es < 5e-2
    assert abs(plastic.max() - 0.162) < 0.01
    S.write_vtk(str(tmp_path / "solution.vtk"))


def _mixed(tmp_path, n, q, order):
    path = str(tmp_path / ("mix_%d.msh" % n))
    gw.write_wellbore_msh(path, n, q, tri_quadrants=(1, 3))
    bcs, mat = gw.reference_bcs()
    return ip.GmshProblem(ip.GmshMesh(path), bcs, order=order, **mat)


@pytest.mark.parametrize("order", [1, 2, 3])
def test_mixed_mesh_bit_exact_with_oracle(tmp_path, order):
    """a mixed triangle/quadrilateral mesh (triangles in the padded block shape)
    through the full-tangent and the initial-stiffness Newton iterations:
    bit-identical to the oracle run on the same element blocks"""
    pb = _mixed(tmp_path, 9, 1.3, order)
    mesh = {k: pb.array(k) for k in ("node_xy", "connects", "fixed", "f0", "df", "dphi", "weight")}
    mesh["order"] = order
    for tangent in (0, 1):
        sm = ip.ElastoPlasticIntPointsStructMatrix(pb)
        prm = po.default_params(4, E=2000.0, nu=0.2, cohesion=5.0, phi_deg=20.0, psi_deg=20.0, sxx0=0.0,
                                syy0=0.0, szz0=0.0, sxy0=0.0)
        P = po.OracleProblem(prm, mesh=mesh)
        assert sm.n_colors == P.n_colors
        sm.set_newton_tangent(tangent)
        ug, uo = np.zeros(sm.neq), np.zeros(sm.neq)
        sg, lg = sm.newton(ug, 1, newton_rtol=1e-12, newton_max_it=5, cg_rtol=1e-10)
        so, lo = P.solve_steps(uo, 1, newton_rtol=1e-12, newton_max_it=5, cg_rtol=1e-10, tangent_mode=tangent)
        assert sg.newton_iters == so.newton_iters and sg.cg_iters == so.cg_iters
        assert np.array_equal(lg, lo) and np.array_equal(ug, uo)
        ghosts = pb.array("fixed").reshape(-1, 2).all(1)
        assert not ug.reshape(-1, 2)[ghosts].any()


def test_mixed_mesh_solution_matches_the_quadrilateral_one(tmp_path):
    """the verification configuration on mesh 1 with two quadrants split into
    triangles (order 2): the wellbore displacement and the plastic radius agree
    with the all-quadrilateral solution of the same mesh"""
    n, q = gw.REFERENCE_MESHES[1]
    res = {}
    for mixed in (False, True):
        pb = _mixed(tmp_path, n, q, 2) if mixed else _problem(tmp_path, n, q)
        sm = ip.ElastoPlasticIntPointsStructMatrix(pb)
        sm.set_preconditioner(ip.PREC_BLOCK_JACOBI)
        u = np.zeros(sm.neq)
        st, _ = sm.newton(u, 1, newton_rtol=1e-9, newton_max_it=60, cg_rtol=1e-10)
        assert st.converged
        xy = pb.array("node_xy").reshape(-1, 2)
        well = np.isclose(np.hypot(xy[:, 0], xy[:, 1]), 0.1, atol=1e-9)
        ur = (u.reshape(-1, 2)[well] * xy[well]).sum(1) / 0.1
        res[mixed] = (ur.mean(), ur.min(), ur.max())
    print("wellbore radial displacement, quadrilaterals %.6e, mixed %.6e (min %.6e max %.6e)"
          % (res[False][0], res[True][0], res[True][1], res[True][2]))
    assert abs(res[True][0] / res[False][0] - 1) < 5e-3
