"""The device's constitutive source (csrc/constitutive.cuh), compiled for the
host with the device's no-contraction rule, against the oracle: every golden
point, with and without the tangent, with the reference's and the consistent
tangent, bit for bit.  The GPU parity tests then only have to show that the
device compiles the same operations (they do: tests/test_gpu_parity.py)."""
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
    L.host_ip_update.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, _dp, _dp, _dp, C.c_double, _dp, _dp,
                                 _dp, _dp, _dp]
    return L


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(os.path.join(HERE, "golden", "constitutive.npz")))


def _host_point(L, g, i, dep, consistent):
    mc = np.array([g["cohesion"][i], g["sinphi"][i], g["cosphi"][i], g["tanphi"][i], g["sinpsi"][i]])
    p6 = g["plastic6"][i]
    pl = np.ascontiguousarray(p6[[0, 1, 3, 5]])
    eps = np.ascontiguousarray(g["strain3"][i])
    sw, s4, p4, d9 = np.zeros(3), np.zeros(4), np.zeros(4), np.zeros(9)
    al = C.c_double()
    mt = L.host_ip_update(int(dep), int(consistent), g["lam"][i], g["mu"][i], po.ptr(mc), po.ptr(eps), po.ptr(pl),
                          g["weight"][i], po.ptr(sw), po.ptr(s4), po.ptr(p4), C.byref(al), po.ptr(d9))
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


@pytest.mark.parametrize("dep,consistent", [(False, 0), (True, 0), (True, 1)],
                         ids=["sigma", "sigma-dep", "sigma-dep-consistent"])
def test_device_source_equals_oracle_on_golden_points(host, gold, dep, consistent):
    n = len(gold["weight"])
    bad = []
    for i in range(n):
        h = _host_point(host, gold, i, dep, consistent)
        if consistent:
            with po.consistent_tangent():
                o = _oracle_point(gold, i, dep)
        else:
            o = _oracle_point(gold, i, dep)
        same = all(_eq(a, b) for a, b in zip(h[:4], o[:4])) and h[4] == o[4]
        if dep:
            same = same and _eq(h[5], o[5])
        if not same:
            bad.append(i)
    assert not bad, "points differing from the oracle: %s" % bad[:10]
    if not dep:
        mt = np.array([_host_point(host, gold, i, False, 0)[4] for i in range(n)])
        assert (mt == 0).sum() > 700 and (mt == 1).sum() > 200 and (mt == -1).sum() > 100
