"""The CPU oracle against the reference's own constitutive code.

Golden vectors: tests/golden/constitutive.npz, produced by
tests/golden/make_golden.py from the reference headers compiled unmodified
(oracle/_ref).  The oracle must reproduce them bit for bit.
"""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import pyoracle as po

GOLD = os.path.join(os.path.dirname(__file__), "golden", "constitutive.npz")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def _mc(g, i):
    m = po.MC()
    m.cohesion, m.sinphi, m.cosphi, m.tanphi, m.sinpsi = (
        g["cohesion"][i], g["sinphi"][i], g["cosphi"][i], g["tanphi"][i], g["sinpsi"][i])
    return m


def _run(g, i, dep, alias=False):
    el = po.Elastic(g["lam"][i], g["mu"][i])
    mc = _mc(g, i)
    s3 = np.ascontiguousarray(g["strain3"][i])
    p6 = np.ascontiguousarray(g["plastic6"][i])
    sw, s6, pout, st6 = np.zeros(3), np.zeros(6), np.zeros(6), np.zeros(6)
    d9 = np.zeros(9) if dep else None
    mt, al = C.c_int(), C.c_double()
    L = po.lib()
    if alias:
        L.orc_ip_update_gpu_alias(C.byref(el), C.byref(mc), po.ptr(s3), po.ptr(p6), g["weight"][i],
                                  po.ptr(sw), po.ptr(s6), po.ptr(pout), C.byref(mt), C.byref(al))
    else:
        L.orc_ip_update(C.byref(el), C.byref(mc), po.ptr(s3), po.ptr(p6), g["weight"][i], po.ptr(sw),
                        po.ptr(d9), po.ptr(s6), po.ptr(pout), po.ptr(st6), C.byref(mt), C.byref(al))
    return sw, d9, s6, pout, mt.value, al.value


def _eq(a, b):
    """bit-level equality up to the sign of zero; NaN equals NaN (the
    reference itself yields NaN for an exactly repeated in-plane eigenvalue,
    FunctionsSpectralDecomp.h:203)"""
    return np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)


def test_golden_covers_every_branch(gold):
    mt = gold["cpu_mtype"]
    assert (mt == 0).sum() > 100 and (mt == 1).sum() > 100 and (mt == -1).sum() > 50


@pytest.mark.parametrize("tag,dep", [("cpu", False), ("cpu_dep", True)])
def test_oracle_bit_exact_vs_reference(gold, tag, dep):
    n = len(gold["lam"])
    bad = []
    for i in range(n):
        sw, d9, s6, pout, mt, al = _run(gold, i, dep)
        ok = (_eq(sw, gold[tag + "_sigma_w3"][i]) and _eq(s6, gold[tag + "_sigma6"][i])
              and _eq(pout, gold[tag + "_plastic6"][i]) and mt == gold[tag + "_mtype"][i]
              and _eq(al, gold[tag + "_alpha"][i]))
        if dep:
            ok = ok and _eq(d9, gold["cpu_dep_dep9"][i])
        if not ok:
            bad.append(i)
    assert not bad, "oracle differs from the reference at points %s" % bad[:10]


def test_reference_gpu_kernel_aliasing_is_reproduced(gold):
    """The reference's residual kernel aliases ProjectSigma's input and output
    (KernelsComputeSigma.h:48); the oracle's aliased variant reproduces it,
    and it differs from the CPU path on some edge/apex points."""
    n = len(gold["lam"])
    for i in range(n):
        sw, _, s6, pout, mt, al = _run(gold, i, False, alias=True)
        assert _eq(s6, gold["gpu_sigma6"][i]) and mt == gold["gpu_mtype"][i]
    a, b = gold["cpu_sigma6"], gold["gpu_sigma6"]
    differ = np.any((a != b) & ~(np.isnan(a) & np.isnan(b)), axis=1)
    assert differ.sum() > 0
    assert np.all(gold["cpu_mtype"][differ] != 0)


def test_sigma_and_sigma_dep_agree(gold):
    """ComputeSigma and ComputeSigmaDep give the same stress bit for bit."""
    assert _eq(gold["cpu_sigma6"], gold["cpu_dep_sigma6"])
    assert np.array_equal(gold["cpu_mtype"], gold["cpu_dep_mtype"])


def _fd_tangent_errors(gold):
    """per return type, max |Dep - dsigma_w/dstrain3| over a point's entries,
    relative to its elastic stiffness w (lambda + 2 mu); central differences
    that stay on the point's branch.  Returns {mtype: [errors]} and the Dep
    matrices of the elastic points."""
    errs, elastic = {0: [], 1: [], -1: []}, []
    g = dict(gold, strain3=gold["strain3"].copy())
    for i in range(len(gold["weight"])):
        s3 = gold["strain3"][i]
        _, d9, _, _, mt, _ = _run(gold, i, True)
        if not np.all(np.isfinite(d9)):
            continue            # repeated in-plane eigenvalue: NaN in the reference too
        h = 1e-7 * max(np.abs(s3).max(), 1e-6)
        F, same = np.zeros((3, 3)), True
        for k in range(3):
            g["strain3"][i] = s3 + h * np.eye(3)[k]
            sp, _, _, _, mp, _ = _run(g, i, True)
            g["strain3"][i] = s3 - h * np.eye(3)[k]
            sm, _, _, _, mm, _ = _run(g, i, True)
            g["strain3"][i] = s3
            same = same and mp == mt and mm == mt
            F[:, k] = (sp - sm) / (2 * h)
        if not same:
            continue
        errs[mt].append(np.abs(d9.reshape(3, 3) - F).max() / (gold["weight"][i] * (gold["lam"][i] + 2 * gold["mu"][i])))
        if mt == 0:
            elastic.append(d9)
    return {k: np.array(v) for k, v in errs.items()}, np.array(elastic)


def test_tangents_against_finite_differences_per_return_type(gold):
    """On the golden points, per return type: the consistent variant of the
    oracle's tangent (orc_set_consistent_tangent) is the derivative of the
    point's weighted stress; the reference's TangentOperator is off by a
    sizeable fraction of the elastic stiffness wherever the point is plastic
    (plane, edge and apex returns) and equal to the consistent one where it is
    elastic."""
    e_ref, d_ref = _fd_tangent_errors(gold)
    with po.consistent_tangent():
        e_con, d_con = _fd_tangent_errors(gold)
    for mt, name in ((1, "plane/edge"), (-1, "apex"), (0, "elastic")):
        print("%-10s n %4d  reference median %.2e max %.2e | consistent median %.2e p90 %.2e"
              % (name, e_ref[mt].size, np.median(e_ref[mt]), e_ref[mt].max(), np.median(e_con[mt]),
                 np.percentile(e_con[mt], 90)))
    assert e_ref[1].size > 200 and e_ref[-1].size > 100 and e_ref[0].size > 700
    assert e_con[1].max() < 1e-6 and np.percentile(e_con[-1], 90) < 1e-6
    assert np.median(e_ref[1]) > 0.05 and np.median(e_ref[-1]) > 0.05
    assert _eq(d_ref, d_con) and np.median(e_con[0]) < 1e-6


# A state of golden point 914 (its material and plastic strain) moved along a
# strain path until an in-plane principal trial stress lies within 7e-7
# (relative) of sigma_zz: 84.97540 against 84.97561.  The point returns to the
# apex, where the projected stress is hydrostatic, c cot(phi) in every
# direction; the reference reconstructs it with eigenvectors that Multiplicity1
# computed one at a time from a nearly singular system, which are far from
# orthogonal here (FunctionsSpectralDecomp.h:116-150, 217-256).
GLITCH = {"lam": 4166.666666666667, "mu": 6250.0, "c": 7.0, "phi": 0.4363323129985824,
          "strain3": [0.010701258239680976, -0.01791932264000126, 0.010302795370944334],
          "plastic6": [0.00036342429229277727, -0.0020668644577720397, 0.0, 0.003073056850626, 0.0,
                       -0.000706630696552844]}


def test_near_repeated_eigenvalue_gives_a_wrong_apex_stress_as_in_the_reference():
    """The oracle keeps the reference's behaviour at a nearly repeated trial
    eigenvalue bit for bit (and against the reference's compiled headers where
    the reference tree is present): the apex stress keeps its trace but is not
    hydrostatic.  (The states 5.4e-6 of strain away on either side along the
    path are hydrostatic to 1e-7: the stress jumps there.)"""
    g = GLITCH
    el = po.Elastic(g["lam"], g["mu"])
    mc = po.MC()
    po.lib().orc_mc_from_angles(g["c"], g["phi"], g["phi"], C.byref(mc))
    s3, p6 = np.array(g["strain3"]), np.array(g["plastic6"])
    sw, s6, pout, st6, d9 = np.zeros(3), np.zeros(6), np.zeros(6), np.zeros(6), np.zeros(9)
    mt, al = C.c_int(), C.c_double()
    po.lib().orc_ip_update(C.byref(el), C.byref(mc), po.ptr(s3), po.ptr(p6), 1.0, po.ptr(sw), po.ptr(d9),
                           po.ptr(s6), po.ptr(pout), po.ptr(st6), C.byref(mt), C.byref(al))
    apex = g["c"] / np.tan(g["phi"])
    assert mt.value == -1
    assert abs((s6[0] + s6[3] + s6[5]) / 3 - apex) < 1e-12 * apex
    assert np.abs(s6[[0, 3, 5]] - apex).max() > 5.0 and abs(s6[1]) > 5.0
    from oracle.build import build_ref
    so = build_ref()
    if so is None:
        pytest.skip("reference tree not present")
    ref = C.CDLL(so)
    P = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    rs6, rsw, rp = np.zeros(6), np.zeros(3), np.zeros(6)
    rmt, ral = C.c_int(), C.c_double()
    ref.ref_ip_sigma(C.c_double(g["lam"]), C.c_double(g["mu"]), C.c_double(g["phi"]), C.c_double(g["phi"]),
                     C.c_double(g["c"]), P(s3), P(p6), C.c_double(1.0), P(rsw), P(rs6), P(rp), C.byref(rmt),
                     C.byref(ral))
    assert rmt.value == -1 and _eq(rs6, s6)
