"""Block-matrix layouts on the host (no GPU): tests/layout_check.cpp, compiled
here with the library's own host sources, checks the FP64 layout (rows sorted
by length) and the FP32 layouts (node order, one slot per lane or slot pairs)
block by block against the nodal pattern, the slot pairs' sectors and the row
stencils; this test reads its summary lines."""
import os
import re
import shutil
import subprocess

import pytest

from intpointsfem_gb300 import build as ipbuild
from intpointsfem_gb300 import gmsh_wellbore as gw

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "intpointsfem_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    inc = os.path.join(ipbuild.cuda_home(), "include")
    if not gxx or not os.path.exists(os.path.join(inc, "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA headers are missing")
    exe = str(tmp_path_factory.mktemp("layout") / "layout_check")
    subprocess.check_call([gxx, "-O2", "-std=c++17", "-pthread", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
                           "-I" + inc, os.path.join(HERE, "layout_check.cpp"), os.path.join(CSRC, "host_setup.cpp"),
                           os.path.join(CSRC, "host_gmsh.cpp"), "-o", exe])
    return exe


def _run(exe, *args):
    p = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0 and "FAIL" not in p.stdout, p.stdout + p.stderr
    out = {}
    for line in p.stdout.splitlines():
        m = re.match(r"(\S+) stencils (\d+) slots (\d+) sectors (\d+)", line)
        if m:
            out[m.group(1)] = tuple(int(x) for x in m.groups()[1:])
        m = re.match(r"fp32-sym stencils (\d+) slots (\d+) sectors (\d+) tstencils (\d+) stored (\d+) lower (\d+)",
                     line)
        if m:
            out["fp32-sym"] = tuple(int(x) for x in m.groups())
    assert {"fp64", "fp32-single", "fp32-pairs"} <= set(out), p.stdout
    return out


@pytest.mark.parametrize("n", [1, 12, 100])
def test_wellbore_layouts(checker, n):
    out = _run(checker, "wellbore", n)
    st = {k: v[0] for k, v in out.items()}
    # the structured grid's rows fall into at most 16 stencils (4 node kinds
    # and their edge variants); every layout finds the same ones
    assert 0 < st["fp64"] <= 16 and st["fp64"] == st["fp32-single"] == st["fp32-pairs"]
    if n >= 12:
        assert st["fp64"] == 16
        # slot pairs: fewer 32-byte sectors of FP32 blocks per SpMV than one slot per lane
        assert out["fp32-pairs"][2] < 0.9 * out["fp32-single"][2]
        # the upper-only layout: 11 upper and 19 transposed stencils, the
        # stored and lower blocks make up the nodal pattern, about half the slots
        ns, slots, _, nt, stored, lower = out["fp32-sym"]
        assert (ns, nt) == (11, 19)
        assert stored + lower == (8 * n + 1) ** 2 and stored - lower == (2 * n + 1) ** 2
        assert slots < 0.55 * out["fp32-pairs"][1]


@pytest.mark.parametrize("order,tri", [(1, ()), (2, ()), (3, ()), (2, (1,))])
def test_gmsh_layouts(checker, tmp_path, order, tri):
    path = str(tmp_path / "w.msh")
    gw.write_wellbore_msh(path, 6, 1.175, tri_quadrants=tri)
    out = _run(checker, "gmsh", path, order)
    if order == 3:
        # vertex rows of 49 blocks are longer than a stencil: explicit columns only
        assert all(v[0] == 0 for v in out.values())
