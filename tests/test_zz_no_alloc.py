"""The allocation-free dot product (ipfem_dot_noalloc) against the context dot.

ipfem_dot_noalloc serves callers that must not allocate device memory: an
application that owns all device memory through its own pool, or a
latency-critical pipeline that must not stall on cudaMalloc (which
synchronises the device).  It keeps its scratch in a fixed array inside the
library instead of in a context, so this file checks, through the C-ABI,
that two consecutive calls give exactly the context dot's result (the same
canonical reduction order, so the comparison is exact), and that a length
beyond the array's capacity is refused.  The file is named to run last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ip = pytest.importorskip("intpointsfem_gb300")

MAX_LEN = 2 * 256 * 65536


def test_dot_noalloc_matches_context_dot_twice():
    torch = pytest.importorskip("torch")
    L = ip.lib()
    w = ip.WellboreMesh(ip.wellbore_params(24))
    sm = ip.ElastoPlasticIntPointsStructMatrix(w)
    rng = np.random.default_rng(11)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        a = torch.tensor(rng.normal(size=sm.neq), dtype=torch.float64, device="cuda")
        b = torch.tensor(rng.normal(size=sm.neq) * (call + 1), dtype=torch.float64, device="cuda")
        out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        expected = sm.dot(a, b)
        st = L.ipfem_dot_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), sm.neq,
                                 C.c_void_p(out.data_ptr()), C.c_void_p(stream))
        torch.cuda.synchronize()
        assert st == 0, L.ipfem_last_error(None).decode()
        assert out.item() == expected
        assert out.item() == pytest.approx(float(np.dot(a.cpu().numpy(), b.cpu().numpy())), rel=1e-12)


def test_dot_noalloc_rejects_oversize_and_odd():
    torch = pytest.importorskip("torch")
    L = ip.lib()
    a = torch.zeros(4, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = L.ipfem_dot_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(a.data_ptr()), MAX_LEN + 2,
                             C.c_void_p(out.data_ptr()), None)
    assert st == 5 and b"maximum" in L.ipfem_last_error(None)
    st = L.ipfem_dot_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(a.data_ptr()), 3, C.c_void_p(out.data_ptr()),
                             None)
    assert st == 5


def test_dot_noalloc_rejects_offset_slice_and_launches_nothing():
    """a vector that starts at an odd double offset of an allocation is
    refused with IPFEM_INVALID; the output is left untouched"""
    torch = pytest.importorskip("torch")
    L = ip.lib()
    base = torch.ones(66, dtype=torch.float64, device="cuda")
    out = torch.full((1,), 7.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    st = L.ipfem_dot_noalloc(C.c_void_p(base[1:].data_ptr()), C.c_void_p(base.data_ptr()), 64,
                             C.c_void_p(out.data_ptr()), None)
    torch.cuda.synchronize()
    assert st == 5 and b"16-byte" in L.ipfem_last_error(None)
    assert out.item() == 7.0
