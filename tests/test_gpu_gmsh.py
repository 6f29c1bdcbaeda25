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


def _problem(tmp_path, n, q, cohesion=5.0):
    path = str(tmp_path / ("wb_%d.msh" % n))
    gw.write_wellbore_msh(path, n, q)
    bcs, mat = gw.reference_bcs(cohesion)
    return ip.GmshProblem(ip.GmshMesh(path), bcs, **mat)


def _oracle(pb, cohesion=5.0):
    prm = po.default_params(4, E=2000.0, nu=0.2, cohesion=cohesion, phi_deg=20.0, psi_deg=20.0, sxx0=0.0,
                            syy0=0.0, szz0=0.0, sxy0=0.0)
    return po.OracleProblem(prm, mesh={k: pb.array(k) for k in ("node_xy", "connects", "fixed", "f0", "df")})


@pytest.mark.parametrize("tangent,accel", [(0, 0), (1, 0), (1, 1)])
def test_gmsh_problem_bit_exact_with_oracle(tmp_path, tangent, accel):
    pb = _problem(tmp_path, 9, 1.3)
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
