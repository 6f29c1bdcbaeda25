"""Semi-analytic Runge-Kutta solution of the hydrostatic wellbore (test
infrastructure only).

Restates TRKSolution::RKProcess and TRKSolution::F (TRKSolution.cpp:99-224)
as driven by RKApproximation (main.cpp:609-659): radial equilibrium of a
plane-strain hole under hydrostatic loading, integrated from the outer radius
re inward to the wellbore radius rw with classical RK4 (or Euler) in the
radial displacement u and the radial stress sigma_rr, the tangent Lame
parameters of each step taken from the elastoplastic tangent of the point
just computed (lambda = Dep(0,5), G = Dep(4,4) / 2, TRKSolution.cpp:189-191).
The point update is the oracle's restatement of the reference's Mohr-Coulomb
return mapping (orc_ip_tangent6), started from a stress- and strain-free
state at every point as the reference's FillPointsMemory does.

Quirks kept from the reference: the state update of point i+1 takes
sigma_rr = sigma_rr(i) + h * dsigma_k1 (an Euler step), and that value, not
the RK4 one, replaces sigma_rr(i+1) (TRKSolution.cpp:167-205).
"""
import ctypes as C

import numpy as np

from . import pyoracle as po

_T6 = None


def _tangent6():
    global _T6
    if _T6 is None:
        L = po.lib()
        f = L.orc_ip_tangent6
        dp = C.POINTER(C.c_double)
        f.argtypes = [C.POINTER(po.Elastic), C.POINTER(po.MC), dp, dp, dp, dp, dp, C.POINTER(C.c_int)]
        f.restype = None
        _T6 = f
    return _T6


def _F(r, ur, sigma_r, lam, G):
    """TRKSolution::F (TRKSolution.cpp:216-224)"""
    sigma_t = (lam * r * sigma_r + 4 * G * (G + lam) * ur) / ((2 * G + lam) * r)
    d_ur = (r * sigma_r - lam * ur) / (r * lam + 2 * G * r)
    d_sigmar = (-sigma_r + sigma_t) / r
    return d_ur, d_sigmar


def rk_process(E, nu, cohesion, phi_deg, psi_deg, rw, re, u_re, sigma_re, n_points, euler=False):
    """rows [n_points][11]: radius, u, sigma rr tt zz, eps rr tt zz, eps_p rr tt zz
    (the columns of the reference's output file)"""
    el = po.Elastic()
    po.lib().orc_lame_from_engineering(E, nu, C.byref(el))
    mc = po.MC()
    po.lib().orc_mc_from_angles(cohesion, np.deg2rad(phi_deg), np.deg2rad(psi_deg), C.byref(mc))
    t6 = _tangent6()
    n = int(n_points)
    h = (rw - re) / n
    r = np.zeros(n + 1)
    u = np.zeros(n + 1)
    srr = np.zeros(n + 1)
    mem_sig = np.zeros((n + 1, 3))
    mem_eps = np.zeros((n + 1, 3))
    mem_epp = np.zeros((n + 1, 3))
    r[0], u[0], srr[0] = re, u_re, sigma_re
    mem_sig[0] = sigma_re
    lam, G = el.lam, el.mu
    strain = (C.c_double * 6)()
    epp0 = (C.c_double * 6)()
    sig6 = (C.c_double * 6)()
    epp6 = (C.c_double * 6)()
    T = (C.c_double * 36)()
    mt = C.c_int()
    for i in range(n):
        du1, ds1 = _F(r[i], u[i], srr[i], lam, G)
        if not euler:
            du2, ds2 = _F(r[i] + h / 2., u[i] + h * du1 / 2., srr[i] + h * ds1 / 2., lam, G)
            du3, ds3 = _F(r[i] + h / 2., u[i] + h * du2 / 2., srr[i] + h * ds2 / 2., lam, G)
            du4, ds4 = _F(r[i] + h, u[i] + h * du3, srr[i] + h * ds3, lam, G)
            r[i + 1] = r[i] + h
            u[i + 1] = u[i] + 1. / 6. * h * (du1 + 2. * du2 + 2. * du3 + du4)
            srr[i + 1] = srr[i] + 1. / 6. * h * (ds1 + 2. * ds2 + 2. * ds3 + ds4)
        else:
            r[i + 1] = r[i] + h
            u[i + 1] = u[i] + h * du1
            srr[i + 1] = srr[i] + h * ds1
        r1, ur1 = r[i + 1], u[i + 1]
        sigma_r = srr[i] + h * ds1
        sigma_t = (lam * r1 * sigma_r + 4 * G * (G + lam) * ur1) / ((2 * G + lam) * r1)
        nu_t = lam / (2.0 * (lam + G))
        Ey = G * (3.0 * lam + 2.0 * G) / (lam + G)
        eps_r = (1 + nu_t) * ((1 - nu_t) * sigma_r - nu_t * sigma_t) / Ey
        eps_t = (1 + nu_t) * ((1 - nu_t) * sigma_t - nu_t * sigma_r) / Ey
        # total strain XX = eps_r, YY = eps_t (order XX XY XZ YY YZ ZZ)
        strain[0], strain[1], strain[2], strain[3], strain[4], strain[5] = eps_r, 0.0, 0.0, eps_t, 0.0, 0.0
        t6(C.byref(el), C.byref(mc), strain, epp0, sig6, epp6, T, C.byref(mt))
        lam = T[0 * 6 + 5]
        G = T[4 * 6 + 4] / 2.0
        mem_sig[i + 1] = (sig6[0], sig6[3], sig6[5])
        mem_eps[i + 1] = (eps_r, eps_t, 0.0)
        mem_epp[i + 1] = (epp6[0], epp6[3], epp6[5])
        srr[i + 1] = sigma_r
    return np.column_stack([r[:n], u[:n], mem_sig[:n], mem_eps[:n], mem_epp[:n]])
