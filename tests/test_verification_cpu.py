"""The reference's own verification of the hydrostatic wellbore problem
(mathematica_notebooks/RK_Verification, written by TRKSolution and by the
classic NeoPZ element loop; fixture tests/golden/rk_verification.npz):

- the oracle's restatement of the Runge-Kutta integration (oracle/orc_rk.py,
  TRKSolution.cpp:99-224) on top of its Mohr-Coulomb return mapping
  reproduces the reference's RK output to its printed precision;
- the oracle's finite-element solution of the same problem agrees with the
  reference's finite-element solution along y = 0."""
import numpy as np
import pytest

from oracle import orc_rk
from oracle import pyoracle as po
from verification_helpers import compare, fixture, problem_kw


@pytest.mark.parametrize("case", ["ep", "el"])
def test_rk_restatement_reproduces_reference_rk_output(case):
    f = fixture()
    rows = orc_rk.rk_process(float(f["E"]), float(f["nu"]), float(f[case + "_cohesion"]), 20.0, 20.0,
                             float(f["rw"]), float(f["re"]), float(f[case + "_u_re"]), float(f[case + "_sigma_re"]),
                             int(f[case + "_n_points"]))
    ref = f[case + "_rows"]
    mine = rows[f[case + "_index"]]
    # radius, u, stresses, total strains; plastic strains where they are not round-off (elastoplastic case)
    cols = list(range(0, 7)) + ([8, 9] if case == "ep" else [])
    for c in cols:
        scale = np.abs(ref[:, c]).max()
        assert np.abs(mine[:, c] - ref[:, c]).max() <= 1e-5 * scale, (case, c)
    if case == "ep":
        # the plastic zone of the reference's RK solution ends at r = 0.1624 m
        plastic = np.abs(mine[:, 8]) > 1e-12
        assert abs(mine[plastic, 0].max() - 0.1624) < 2e-3


@pytest.mark.parametrize("case,cohesion", [("ep", 5.0), ("el", 1.0e10)])
def test_oracle_fem_matches_reference_fem(case, cohesion):
    n = 20
    P = po.OracleProblem(po.default_params(n, **problem_kw(cohesion)), nthreads=0)
    u = np.zeros(P.neq)
    st, _ = P.solve_steps(u, 10, newton_max_it=60)
    assert st.converged
    sg = P.arr("sigma").reshape(-1, 6)
    err = compare(n, u, P.arr("node_xy"), P.arr("connects"), sg[:, 0], sg[:, 1], sg[:, 3], sg[:, 5],
                  P.arr("mtype"), fixture()[case + "_fem"])
    assert err["u"] < 1e-2, err
    assert max(err["s_rr"], err["s_tt"], err["s_zz"]) < 6e-2, err
    if case == "ep":
        assert abs(err["plastic_radius"] - 0.1624) < 0.01, err
    else:
        assert err["plastic_radius"] == 0.0
