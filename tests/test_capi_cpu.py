"""Host-side checks of the C-ABI library (no GPU needed): it loads, exports
every entry point include/ipfem.h declares, and its host logic (mesh
provider, colouring, argument validation) agrees with the oracle."""
import os
import re

import numpy as np
import pytest

import intpointsfem_gb300 as ip
from oracle import pyoracle as po

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "ipfem.h")


def declared_symbols():
    txt = open(HDR).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ipfem_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    names = declared_symbols()
    assert len(names) >= 25
    L = ip.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_no_device_is_reported_not_faked():
    """without a GPU, creating a context fails loudly (no CPU fallback)"""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    w = ip.WellboreMesh(ip.wellbore_params(4))
    with pytest.raises(ip.IpfemError) as e:
        ip.ElastoPlasticIntPointsStructMatrix(w)
    assert e.value.status == 7


@pytest.mark.parametrize("n,mode", [(5, 0), (12, 2), (40, 1)])
def test_mesh_provider_equals_oracle(n, mode):
    w = ip.WellboreMesh(ip.wellbore_params(n, material_mode=mode))
    P = po.OracleProblem(po.default_params(n, material_mode=mode), nthreads=2)
    assert np.array_equal(w.array("node_xy"), P.arr("node_xy"))
    assert np.array_equal(w.array("connects"), P.arr("connects"))
    assert np.array_equal(w.array("fixed"), P.arr("fixed"))
    assert np.array_equal(w.array("f0"), P.arr("f0"))
    assert np.array_equal(w.array("df"), P.arr("df"))
    assert np.array_equal(w.array("weight"), P.arr("weight"))
    B = P.arr("B").reshape(-1, 9, 3, 18)
    dn = w.array("dphi").reshape(-1, 9, 2, 9)
    assert np.array_equal(dn[:, :, 0, :], B[:, :, 0, 0::2])
    assert np.array_equal(dn[:, :, 1, :], B[:, :, 1, 0::2])
    # structural zeros and duplicated entries of the reference block layout
    assert np.all(B[:, :, 0, 1::2] == 0) and np.all(B[:, :, 2, 0::2] == 0)
    assert np.array_equal(B[:, :, 1, 1::2], B[:, :, 0, 0::2]) and np.array_equal(B[:, :, 2, 1::2], B[:, :, 1, 0::2])
    m = P.mats()
    if mode >= 1:
        assert np.array_equal(w.array("el_cohesion"), m[:, 0])
    if mode >= 2:
        assert np.allclose(np.sin(w.array("el_phi")), m[:, 1], rtol=0, atol=2e-16)


def test_coloring_known_answer_3x3():
    """hand-derived greedy colouring of a 3x3 structured quad grid
    (elements numbered radial-fastest): pass 0 takes (even i, even j), pass 1
    (odd i, even j), pass 2 (even i, odd j), pass 3 the centre"""
    w = ip.WellboreMesh(ip.wellbore_params(3))
    nc, col = ip.color_elements(w.array("connects"), w.n_nodes)
    assert nc == 4
    assert col.tolist() == [0, 1, 0, 2, 3, 2, 0, 1, 0]


@pytest.mark.parametrize("n", [1, 2, 7, 40])
def test_coloring_product_equals_oracle_and_is_valid(n):
    w = ip.WellboreMesh(ip.wellbore_params(n))
    nc, col = ip.color_elements(w.array("connects"), w.n_nodes)
    P = po.OracleProblem(po.default_params(n), nthreads=1)
    assert nc == P.n_colors and np.array_equal(col, P.arr("el_color"))
    assert nc == (1 if n == 1 else 4)
    con = w.array("connects").reshape(-1, 9)
    for c in range(nc):
        nodes = con[col == c].ravel()
        assert len(nodes) == len(set(nodes.tolist())), "two same-coloured elements share a connect"


def test_coloring_rejects_bad_connects():
    con = np.zeros(9, np.int32)
    con[3] = 99
    with pytest.raises(ip.IpfemError):
        ip.color_elements(con, 10)


def test_wellbore_rejects_bad_params():
    with pytest.raises(ip.IpfemError):
        ip.WellboreMesh(ip.wellbore_params(0))


def test_dot_noalloc_rejects_bad_arguments_before_any_device_call():
    """ipfem_dot_noalloc validates every argument before its first CUDA call,
    so these rejections need no GPU: the addresses are never dereferenced.
    A slice at an odd double offset (8 bytes past a 16-byte boundary) is
    refused, as are null pointers, odd lengths and lengths past the
    maximum."""
    import ctypes as C

    L = ip.lib()
    a, b, out = 0x10000, 0x20000, 0x30000          # 16-byte aligned, never dereferenced
    cases = [
        (a + 8, b, 16, out, b"16-byte"),           # d_a at an odd double offset
        (a, b + 8, 16, out, b"16-byte"),
        (a, b, 16, out + 4, b"8-byte"),            # d_out not a double address
        (0, b, 16, out, b"null"),
        (a, b, 3, out, b"odd"),
        (a, b, 2 * 256 * 65536 + 2, out, b"maximum"),
    ]
    for pa, pb, n, po_, msg in cases:
        st = L.ipfem_dot_noalloc(C.c_void_p(pa), C.c_void_p(pb), n, C.c_void_p(po_), None)
        assert st == 5, (pa, pb, n, po_)
        assert msg in L.ipfem_last_error(None), L.ipfem_last_error(None)


def test_struct_matrix_class_compiles_links_and_throws_without_device(tmp_path):
    """the C++ class of include/ipfem_pz.hpp compiles with g++ -Wall -Werror,
    links against libipfem.so, refuses a bad element order, and (without a
    GPU) throws std::runtime_error from its constructor with the library's
    message, as the reference's struct matrix throws on CUDA failures"""
    import subprocess

    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present (the GPU test drives the class)")
    except ImportError:
        pass
    from struct_matrix_build import build_driver

    exe = build_driver(tmp_path)
    r = subprocess.run([exe, "6", "0.5", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 3, (r.stdout, r.stderr)
    assert "runtime_error: ipfem: no sm_103 device" in r.stdout, r.stdout
