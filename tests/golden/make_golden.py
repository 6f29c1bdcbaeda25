"""Generate tests/golden/constitutive.npz from the reference's own code.

The reference's constitutive headers (FunctionsStressStrain.h,
FunctionsTangentOperator.h and the headers they include) are compiled
unmodified by oracle/build.py into oracle/_ref/libipfem_ref.so, and driven
through three per-point sequences of the reference:

  cpu      TPZConstitutiveLawProcessor.cpp:163-195  (ComputeSigma, CPU)
  cpu_dep  TPZConstitutiveLawProcessor.cpp:377-423  (ComputeSigmaDep, CPU)
  gpu      KernelsComputeSigma.h:7-74               (ComputeSigmaKernel)

Inputs are seeded synthetic (strain, committed plastic strain, material)
triples chosen to visit every branch: elastic, main plane, right and left
edge, apex, repeated eigenvalues, zero strain, and in-situ seeded states.
The trigonometric values the reference evaluates (sin/cos/tan of phi, psi)
are stored with the inputs so that the checks do not depend on the libm of
the machine running them.

Run from the repository root:  python tests/golden/make_golden.py
"""
import ctypes as C
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import build as obuild  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "constitutive.npz")


def main():
    so = obuild.build_ref()
    if so is None:
        raise SystemExit("reference tree not found; set IPFEM_REFERENCE_DIR")
    ref = C.CDLL(so)
    dp = C.POINTER(C.c_double)

    def P(a):
        return a.ctypes.data_as(dp)

    rng = np.random.default_rng(20260101)
    cases = []

    def lame(E, nu):
        return (E * nu) / ((1.0 + nu) * (1.0 - 2.0 * nu)), E / (2.0 * (1.0 + nu))

    mats = [(15000.0, 0.2, 10.0, 30.0), (2000.0, 0.2, 5.0, 20.0), (15000.0, 0.2, 7.0, 25.0),
            (15000.0, 0.25, 14.0, 35.0)]
    # in-situ seed of the wellbore problem: -C^{-1} sigma0 (sigma0 = -40, -50, zz = -18)
    n_rand = 1200
    for t in range(n_rand):
        E, nu, c, phideg = mats[t % len(mats)]
        lam, mu = lame(E, nu)
        scale = 10.0 ** rng.uniform(-4.5, -1.8)
        kind = t % 6
        s3 = rng.normal(size=3) * scale
        p6 = np.zeros(6)
        if kind == 1:                    # repeated in-plane eigenvalue
            s3[2] = s3[0]
            s3[1] = 0.0
        elif kind == 2:                  # tensile volumetric (apex side)
            s3[0] = abs(s3[0]) + scale
            s3[2] = abs(s3[2]) + scale
        elif kind == 3:                  # pure shear
            s3[0] = 0.0
            s3[2] = 0.0
        if t % 3 != 0:                   # committed plastic strain, plane-strain pattern
            p6[[0, 1, 3, 5]] = rng.normal(size=4) * scale * 0.3
        if t % 5 == 0:                   # in-situ seeded
            K = lam + 2 * mu / 3
            sig0 = np.array([-40.0, 0.0, 0.0, -50.0, 0.0, -18.0])
            a1 = (lam + mu) / (3 * lam * mu + 2 * mu * mu)
            a2 = lam / (6 * lam * mu + 4 * mu * mu)
            e = np.zeros(6)
            e[0] = a1 * sig0[0] - a2 * (sig0[3] + sig0[5])
            e[3] = a1 * sig0[3] - a2 * (sig0[0] + sig0[5])
            e[5] = a1 * sig0[5] - a2 * (sig0[3] + sig0[0])
            p6 = -e
            del K
        cases.append((lam, mu, c, math.radians(phideg), s3, p6, float(rng.uniform(0.01, 3.0))))
    # exact special points
    lam, mu = lame(15000.0, 0.2)
    for s3 in ([0.0, 0.0, 0.0], [1e-3, 0.0, 1e-3], [-1e-3, 0.0, -1e-3], [0.0, 2e-3, 0.0], [5e-3, 0.0, 5e-3]):
        cases.append((lam, mu, 10.0, math.radians(30.0), np.array(s3, float), np.zeros(6), 1.0))

    n = len(cases)
    inp = {k: np.zeros(s) for k, s in (("lam", n), ("mu", n), ("cohesion", n), ("phi", n), ("psi", n),
                                         ("sinphi", n), ("cosphi", n), ("tanphi", n), ("sinpsi", n),
                                         ("weight", n), ("strain3", (n, 3)), ("plastic6", (n, 6)))}
    out = {}
    for tag in ("cpu", "cpu_dep", "gpu"):
        out[tag + "_sigma_w3"] = np.zeros((n, 3))
        out[tag + "_sigma6"] = np.zeros((n, 6))
        out[tag + "_plastic6"] = np.zeros((n, 6))
        out[tag + "_mtype"] = np.zeros(n, np.int32)
        out[tag + "_alpha"] = np.zeros(n)
    out["cpu_dep_dep9"] = np.zeros((n, 9))
    for i, (lam, mu, c, phi, s3, p6, w) in enumerate(cases):
        psi = phi
        inp["lam"][i], inp["mu"][i], inp["cohesion"][i], inp["phi"][i], inp["psi"][i] = lam, mu, c, phi, psi
        inp["sinphi"][i], inp["cosphi"][i], inp["tanphi"][i], inp["sinpsi"][i] = (
            math.sin(phi), math.cos(phi), math.tan(phi), math.sin(psi))
        inp["weight"][i] = w
        inp["strain3"][i] = s3
        inp["plastic6"][i] = p6
        s3c = np.ascontiguousarray(s3, dtype=np.float64)
        p6c = np.ascontiguousarray(p6, dtype=np.float64)
        for tag in ("cpu", "cpu_dep", "gpu"):
            sw, s6, po = np.zeros(3), np.zeros(6), np.zeros(6)
            mt, al = C.c_int(), C.c_double()
            args = [C.c_double(lam), C.c_double(mu), C.c_double(phi), C.c_double(psi), C.c_double(c),
                    P(s3c), P(p6c), C.c_double(w), P(sw)]
            if tag == "cpu":
                ref.ref_ip_sigma(*args, P(s6), P(po), C.byref(mt), C.byref(al))
            elif tag == "gpu":
                ref.ref_ip_sigma_gpu(*args, P(s6), P(po), C.byref(mt), C.byref(al))
            else:
                d9 = np.zeros(9)
                ref.ref_ip_sigma_dep(*args, P(d9), P(s6), P(po), C.byref(mt), C.byref(al))
                out["cpu_dep_dep9"][i] = d9
            out[tag + "_sigma_w3"][i] = sw
            out[tag + "_sigma6"][i] = s6
            out[tag + "_plastic6"][i] = po
            out[tag + "_mtype"][i] = mt.value
            out[tag + "_alpha"][i] = al.value
    np.savez_compressed(OUT, **inp, **out)
    mt = out["cpu_mtype"]
    diff = int(np.sum(np.any(out["cpu_sigma6"] != out["gpu_sigma6"], axis=1)))
    print("wrote", OUT, "points", n, "mtype counts", {int(k): int((mt == k).sum()) for k in (-1, 0, 1)},
          "cpu/gpu-kernel sequence differ at", diff)


if __name__ == "__main__":
    main()
