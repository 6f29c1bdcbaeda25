"""Writes tests/golden/rk_verification.npz from the reference's own
verification output in mathematica_notebooks/RK_Verification/:

- *RKdata.txt, written by TRKSolution::RKProcess (TRKSolution.cpp:99-214)
  as driven by main.cpp:374-446 and 609-659;
- *FEMdata.csv, the reference's finite-element solution of the same problem
  (classic NeoPZ element loop, L2-projected post-processing, main.cpp:289-324)
  sampled along the ray y = 0 from r = 0.1 m to 4 m.

Each file lists, from r = 4 m inward to r = 0.1 m, the radius, the radial
displacement, sigma_rr, sigma_tt, sigma_zz, the total and the plastic strain
(rr, tt, zz) of the hydrostatic wellbore problem integrated by fourth-order
Runge-Kutta.  The fixture keeps the inputs of the integration and every 20th
row of the elastoplastic case (every 10th of the elastic one) plus the last
row, with the row indices.

    python tests/golden/make_rk_fixture.py [reference root]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load(path):
    return np.loadtxt(path, skiprows=1)


def load_fem(path):
    """arc-ordered rows: x, u_x, sigma xx yy zz, plastic strain xx yy"""
    import csv
    with open(path) as fh:
        rows = list(csv.reader(fh))
    h = rows[0]
    cols = ["Points:0", "Displacement:0", "Stress:0", "Stress:4", "Stress:8", "StrainPlastic:0", "StrainPlastic:4"]
    idx = [h.index(c) for c in cols]
    return np.array([[float(r[i]) for i in idx] for r in rows[1:]])


# the reference tree: argument, IPFEM_REFERENCE_DIR, or `reference` beside the repository root
DEFAULT_REF = os.environ.get("IPFEM_REFERENCE_DIR") or os.path.normpath(
    os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "..", "..", "reference"))


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REF
    d = os.path.join(ref, "mathematica_notebooks", "RK_Verification")
    ep = load(os.path.join(d, "ElastoPlasticRKdata.txt"))
    el = load(os.path.join(d, "ElasticRKdata.txt"))
    fem_ep = load_fem(os.path.join(d, "ElastoPlasticFEMdata.csv"))
    fem_el = load_fem(os.path.join(d, "ElasticFEMdata.csv"))
    ie = np.unique(np.r_[np.arange(0, len(ep), 20), len(ep) - 1])
    il = np.unique(np.r_[np.arange(0, len(el), 10), len(el) - 1])
    np.savez_compressed(
        os.path.join(HERE, "rk_verification.npz"),
        # elastoplastic case: E 2000, nu 0.2, c 5, phi = psi = 20 deg (main.cpp:381-392)
        ep_rows=ep[ie], ep_index=ie, ep_n_points=len(ep), ep_u_re=2.14094e-05, ep_sigma_re=-0.0062899,
        ep_cohesion=5.0,
        # elastic case: cohesion 1e10 (main.cpp:386-388)
        el_rows=el[il], el_index=il, el_n_points=len(el), el_u_re=2.54403e-05, el_sigma_re=0.00124267,
        el_cohesion=1.0e10,
        E=2000.0, nu=0.2, phi_deg=20.0, rw=0.1, re=4.0,
        # the reference's finite-element solutions along y = 0 (every 5th sample + the last)
        ep_fem=fem_ep[np.unique(np.r_[np.arange(0, len(fem_ep), 5), len(fem_ep) - 1])],
        el_fem=fem_el[np.unique(np.r_[np.arange(0, len(fem_el), 5), len(fem_el) - 1])])
    print("rows", len(ie), len(il))


if __name__ == "__main__":
    main()
