"""Shared by the verification tests: the reference's RK / FEM verification
data (tests/golden/rk_verification.npz, written by make_rk_fixture.py) and
the comparison of a finite-element solution of the same hydrostatic wellbore
problem along radial lines."""
import os

import numpy as np

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rk_verification.npz")

# the reference's verification material and loading (main.cpp:374-446): E 2000, nu 0.2,
# c 5 (elastic case: 1e10), phi = psi = 20 deg, stress-free rock, wellbore traction -10
def problem_kw(cohesion):
    return dict(E=2000.0, nu=0.2, cohesion=cohesion, phi_deg=20.0, psi_deg=20.0, sxx0=0.0, syy0=0.0, szz0=0.0,
                sxy0=0.0, pw_final=-10.0)


def fixture():
    return np.load(FIXTURE)


_G = np.sqrt(0.6)
_GP = np.array([-_G, 0.0, _G])
_LOC = [(0, 0), (2, 0), (2, 2), (0, 2), (1, 0), (2, 1), (1, 2), (0, 1), (1, 1)]   # v0..v3, e4..e7, c8


def _l(a, t):
    return (t * (t - 1) / 2, 1 - t * t, t * (t + 1) / 2)[a]


def ip_xy(connects, node_xy):
    """coordinates of the 3x3 Gauss points (q = 3*i_eta + i_xi) of Q2 elements"""
    con = np.asarray(connects).reshape(-1, 9)
    xy = np.asarray(node_xy).reshape(-1, 2)
    out = np.zeros((con.shape[0], 9, 2))
    for q in range(9):
        N = np.array([_l(a, _GP[q % 3]) * _l(b, _GP[q // 3]) for a, b in _LOC])
        out[:, q] = np.einsum("k,ekd->ed", N, xy[con])
    return out.reshape(-1, 2)


def compare(n, u, node_xy, connects, sxx, sxy, syy, szz, mtype, fem):
    """errors of a solution against the reference FEM profile fem[:, (r, u_r,
    s_rr, s_tt, s_zz, ...)]: displacement on y = 0 relative to max|u_r|,
    stresses at integration points beyond the first element layer relative to
    max|s_rr|, and the largest radius of a plastic integration point"""
    xy = np.asarray(node_xy).reshape(-1, 2)
    ray = np.arange(2 * n + 1)
    eu = np.abs(u[2 * ray] - np.interp(xy[ray, 0], fem[:, 0], fem[:, 1])).max() / np.abs(fem[:, 1]).max()
    pts = ip_xy(connects, node_xy)
    rr = np.hypot(pts[:, 0], pts[:, 1])
    th = np.arctan2(pts[:, 1], pts[:, 0])
    c, s = np.cos(th), np.sin(th)
    srr = sxx * c * c + syy * s * s + 2 * sxy * s * c
    stt = sxx * s * s + syy * c * c - 2 * sxy * s * c
    sc = np.abs(fem[:, 2]).max()
    inner = rr > 0.12
    err = {"u": eu}
    for name, v, col in (("s_rr", srr, 2), ("s_tt", stt, 3), ("s_zz", szz, 4)):
        err[name] = np.abs(v - np.interp(rr, fem[:, 0], fem[:, col]))[inner].max() / sc
    plastic = np.asarray(mtype) != 0
    err["plastic_radius"] = rr[plastic].max() if plastic.any() else 0.0
    return err
