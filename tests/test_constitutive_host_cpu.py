"""The device's constitutive source (csrc/constitutive.cuh), compiled for the
host with the device's no-contraction rule, against the oracle: every golden
point, with and without the tangent, with the reference's and the consistent
tangent, with the reference's and the closed-form plane-strain spectral
decomposition, bit for bit; and states next to a nearly repeated eigenvalue.
The GPU parity tests then only have to show that the device compiles the same
operations (they do: tests/test_gpu_parity.py)."""
import contextlib
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from oracle import pyoracle as po

HERE = os.path.dirname(os.path.abspath(__file__))
_dp = C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("host") / "libconstitutive_host.so")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-Wall", "-Werror",
                           "-Wno-unknown-pragmas", os.path.join(HERE, "constitutive_host.cpp"), "-o", so])
    L = C.CDLL(so)
    L.host_ip_update.restype = C.c_int
    L.host_ip_update.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _dp, _dp, _dp, C.c_double, _dp,
                                 _dp, _dp, _dp, _dp]
    return L


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(os.path.join(HERE, "golden", "constitutive.npz")))


def _host_point(L, g, i, dep, consistent, spectral=0):
    mc = np.array([g["cohesion"][i], g["sinphi"][i], g["cosphi"][i], g["tanphi"][i], g["sinpsi"][i]])
    p6 = g["plastic6"][i]
    pl = np.ascontiguousarray(p6[[0, 1, 3, 5]])
    eps = np.ascontiguousarray(g["strain3"][i])
    sw, s4, p4, d9 = np.zeros(3), np.zeros(4), np.zeros(4), np.zeros(9)
    al = C.c_double()
    mt = L.host_ip_update(int(dep), int(consistent), int(spectral), g["lam"][i], g["mu"][i], po.ptr(mc),
                          po.ptr(eps), po.ptr(pl), g["weight"][i], po.ptr(sw), po.ptr(s4), po.ptr(p4), C.byref(al),
                          po.ptr(d9))
    return sw, s4, p4, al.value, mt, d9


def _oracle_point(g, i, dep):
    el = po.Elastic(g["lam"][i], g["mu"][i])
    m = po.MC()
    m.cohesion, m.sinphi, m.cosphi, m.tanphi, m.sinpsi = (
        g["cohesion"][i], g["sinphi"][i], g["cosphi"][i], g["tanphi"][i], g["sinpsi"][i])
    s3 = np.ascontiguousarray(g["strain3"][i])
    p6 = np.ascontiguousarray(g["plastic6"][i])
    sw, s6, pout, st6 = np.zeros(3), np.zeros(6), np.zeros(6), np.zeros(6)
    d9 = np.zeros(9) if dep else None
    mt, al = C.c_int(), C.c_double()
    po.lib().orc_ip_update(C.byref(el), C.byref(m), po.ptr(s3), po.ptr(p6), g["weight"][i], po.ptr(sw),
                           po.ptr(d9), po.ptr(s6), po.ptr(pout), po.ptr(st6), C.byref(mt), C.byref(al))
    return sw, s6[[0, 1, 3, 5]], pout[[0, 1, 3, 5]], al.value, mt.value, d9


def _eq(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)


@contextlib.contextmanager
def _oracle_modes(consistent, spectral):
    with contextlib.ExitStack() as st:
        if consistent:
            st.enter_context(po.consistent_tangent())
        if spectral:
            st.enter_context(po.plane_spectral())
        yield


def _differing(L, g, idx, dep, consistent, spectral):
    bad = []
    for i in idx:
        h = _host_point(L, g, i, dep, consistent, spectral)
        with _oracle_modes(consistent, spectral):
            o = _oracle_point(g, i, dep)
        same = all(_eq(a, b) for a, b in zip(h[:4], o[:4])) and h[4] == o[4]
        if dep:
            same = same and _eq(h[5], o[5])
        if not same:
            bad.append(i)
    return bad


MODES = [(False, 0, 0), (True, 0, 0), (True, 1, 0), (False, 0, 1), (True, 0, 1), (True, 1, 1)]
MODE_IDS = ["sigma", "sigma-dep", "sigma-dep-consistent", "plane-sigma", "plane-sigma-dep",
            "plane-sigma-dep-consistent"]


@pytest.mark.parametrize("dep,consistent,spectral", MODES, ids=MODE_IDS)
def test_device_source_equals_oracle_on_golden_points(host, gold, dep, consistent, spectral):
    n = len(gold["weight"])
    bad = _differing(host, gold, range(n), dep, consistent, spectral)
    assert not bad, "points differing from the oracle: %s" % bad[:10]
    if not dep:
        mt = np.array([_host_point(host, gold, i, False, 0, spectral)[4] for i in range(n)])
        assert (mt == 0).sum() > 700 and (mt == 1).sum() > 200 and (mt == -1).sum() > 100


@pytest.mark.parametrize("dep,consistent,spectral", MODES, ids=MODE_IDS)
def test_device_source_equals_oracle_next_to_a_repeated_eigenvalue(host, dep, consistent, spectral):
    """400 strains within 1e-9 to 1e-5 (relative) of a state whose in-plane
    and out-of-plane trial eigenvalues nearly coincide (the state of
    tests/test_oracle_golden.py::GLITCH): every branch of the reference's
    decomposition near a double root, and the closed form there"""
    from test_oracle_golden import GLITCH

    rng = np.random.default_rng(7)
    s3 = np.array(GLITCH["strain3"])
    n = 400
    scale = np.logspace(-9, -5, n) * np.abs(s3).max()
    dirs = rng.normal(size=(n, 3))
    dirs /= np.linalg.norm(dirs, axis=1)[:, None]
    phi = GLITCH["phi"]
    g = {"lam": np.full(n, GLITCH["lam"]), "mu": np.full(n, GLITCH["mu"]), "cohesion": np.full(n, GLITCH["c"]),
         "sinphi": np.full(n, np.sin(phi)), "cosphi": np.full(n, np.cos(phi)), "tanphi": np.full(n, np.tan(phi)),
         "sinpsi": np.full(n, np.sin(phi)), "weight": np.full(n, 0.25),
         "strain3": s3[None, :] + scale[:, None] * dirs, "plastic6": np.tile(GLITCH["plastic6"], (n, 1))}
    bad = _differing(host, g, range(n), dep, consistent, spectral)
    assert not bad, "states differing from the oracle: %s" % bad[:10]


@pytest.mark.parametrize("dep,consistent,spectral", MODES, ids=MODE_IDS)
def test_device_source_equals_oracle_in_a_random_state(host, dep, consistent, spectral):
    """Every point of a 16 x 16 mesh with heterogeneous material at a random
    displacement (the state tests/test_gpu_parity.py assembles): trial
    stresses up to a thousand times the cohesion, where the reference's choice
    between edge and apex returns turns on rounding, so any difference in the
    operations would show"""
    P = po.OracleProblem(po.default_params(16, material_mode=2), nthreads=2)
    rng = np.random.default_rng(49)
    u = rng.normal(size=P.neq) * 2e-3
    u[P.arr("fixed").astype(bool)] = 0.0
    P.assemble_residual(u, 0.7)
    prm = po.default_params(16, material_mode=2)
    el = po.Elastic()
    po.lib().orc_lame_from_engineering(prm.E, prm.nu, C.byref(el))
    n, npts, M = P.n_ip, 9, P.mats()
    g = {"lam": np.full(n, el.lam), "mu": np.full(n, el.mu), "weight": P.arr("weight").copy(),
         "strain3": P.arr("strain").reshape(n, 3).copy(), "plastic6": P.arr("eps_p").reshape(n, 6).copy()}
    for k, name in enumerate(("cohesion", "sinphi", "cosphi", "tanphi", "sinpsi")):
        g[name] = np.repeat(M[:, k], npts)
    P.close()
    bad = _differing(host, g, range(n), dep, consistent, spectral)
    assert not bad, "points differing from the oracle: %s" % bad[:10]
