"""Shared by the Gmsh replay tests: the reference's logged Newton runs
(tests/golden/reference_logs.json, written by make_log_fixture.py from the
reference's Results logs) and their comparison with a run of ours on the same
mesh and problem.

The logged runs are the initial-stiffness iteration (K assembled once, only
the residual per iteration; with modified-Thomas acceleration in the
*_MODIFIED folders) of the verification configuration on the order-2
wellbore meshes.  Residual norms depend on the shape-function basis (NeoPZ's
hierarchical H1 functions against our Lagrange functions), but the iterates
are the same finite-element functions in any basis, so the ratio of
successive residual norms is basis-independent; its limit is the spectral
radius of I - K0^-1 K_t at the solution."""
import json
import os

import numpy as np

LOGS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_logs.json")


def reference_run(name):
    with open(LOGS) as f:
        return json.load(f)["runs"][name]


def ratios(res):
    r = np.asarray(res, dtype=np.float64)
    return r[1:] / r[:-1]


def iterations_for_reduction(res, factor):
    """iterations until the residual (after iteration 1) has dropped by `factor`"""
    r = np.asarray(res, dtype=np.float64)
    hit = np.nonzero(r <= r[0] * factor)[0]
    return int(hit[0]) + 1 if hit.size else None


def compare(ours, ref, n_ratios):
    ref = np.asarray(ref, dtype=np.float64)
    """(max |ratio difference| over the first 3 ratios, over ratios 4..n, and
    iterations of ours / of the reference to the reference's total reduction)"""
    ro, rr = ratios(ours), ratios(ref)
    n = min(n_ratios, ro.size, rr.size)
    early = np.abs(ro[:3] - rr[:3]).max()
    late = np.abs(ro[3:n] - rr[3:n]).max() if n > 3 else 0.0
    red = ref[-1] / ref[0]
    return early, late, iterations_for_reduction(ours, red), iterations_for_reduction(ref, red)
