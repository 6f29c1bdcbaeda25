"""The reference's own verification problem (hydrostatic wellbore, stress-free
rock, E 2000, nu 0.2, c 5, phi = psi = 20 deg, wellbore traction -10;
main.cpp:374-446) solved on the GPU with the plain FP64 method and with the
chosen method (mixed precision + the shipped learned preconditioner), against
the reference's finite-element solution along y = 0 and the plastic radius of
its Runge-Kutta solution (fixture tests/golden/rk_verification.npz)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ip = pytest.importorskip("intpointsfem_gb300")
from verification_helpers import compare, fixture, problem_kw  # noqa: E402


@pytest.mark.parametrize("method", ["plain", "chosen"])
def test_verification_problem_matches_reference_fem(method):
    from intpointsfem_gb300 import train_preconditioner as tp
    n = 80
    w = ip.WellboreMesh(ip.wellbore_params(n, **problem_kw(5.0)))
    sm = ip.ElastoPlasticIntPointsStructMatrix(w)
    cg_rtol = 1e-8
    if method == "chosen":
        sm.set_precision(ip.MIXED)
        sm.set_node_grid(2 * n + 1, 2 * n + 1)
        sm.mlp_init(0)
        sm.set_mlp_params(tp.load_weights())
        sm.set_preconditioner(ip.PREC_MLP)
        cg_rtol = 1e-4
    u = np.zeros(sm.neq)
    st, _ = sm.newton(u, 10, newton_max_it=60, cg_rtol=cg_rtol)
    assert st.converged and st.fcg_fallbacks == 0
    sg = sm.get_state(1).reshape(4, -1)           # xx, xy, yy, zz
    err = compare(n, u, w.array("node_xy"), w.array("connects"), sg[0], sg[1], sg[2], sg[3], sm.get_state(3),
                  fixture()["ep_fem"])
    print("%s 80x80 vs reference FEM: u %.2e, s_rr %.2e, s_tt %.2e, s_zz %.2e, plastic radius %.4f (RK 0.1624)"
          % (method, err["u"], err["s_rr"], err["s_tt"], err["s_zz"], err["plastic_radius"]))
    assert err["u"] < 1e-2, err
    assert max(err["s_rr"], err["s_tt"], err["s_zz"]) < 5e-2, err
    assert abs(err["plastic_radius"] - 0.1624) < 5e-3, err
