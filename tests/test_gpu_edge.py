"""Edge cases and error behaviour of the C-ABI on the GPU (compared with the
oracle where a result exists)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ip = pytest.importorskip("intpointsfem_gb300")
torch = pytest.importorskip("torch")
from oracle import pyoracle as po  # noqa: E402


def _eq(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)


def test_reference_block_storage_input_equals_compact_input():
    """ipfem_mesh.block_storage (the reference's 27 x 18 fStorage blocks)
    gives the same context as the compact derivative form."""
    n = 10
    w = ip.WellboreMesh(ip.wellbore_params(n, material_mode=2))
    P = po.OracleProblem(po.default_params(n, material_mode=2), nthreads=0)
    B = np.ascontiguousarray(P.arr("B"))
    m = ip.Mesh()
    C.memmove(C.byref(m), C.byref(w.mesh), C.sizeof(ip.Mesh))
    m.dphi = None
    m.block_storage = B.ctypes.data_as(C.POINTER(C.c_double))
    a = ip.ElastoPlasticIntPointsStructMatrix(m, w.material, keep=(w, B))
    b = ip.ElastoPlasticIntPointsStructMatrix(w)
    assert np.array_equal(a.get_setup(3), b.get_setup(3))
    u = np.random.default_rng(0).normal(size=a.neq) * 1e-3
    a.SetLoadFactor(0.4)
    b.SetLoadFactor(0.4)
    assert _eq(a.assemble_residual(u, np.zeros(a.neq)), b.assemble_residual(u, np.zeros(b.neq)))
    # a corrupted block (non-zero structural zero) is rejected
    B2 = B.copy()
    B2[1] = 1.0
    m.block_storage = B2.ctypes.data_as(C.POINTER(C.c_double))
    with pytest.raises(ip.IpfemError) as e:
        ip.ElastoPlasticIntPointsStructMatrix(m, w.material, keep=(w, B2))
    assert e.value.status == 5


def test_newton_heterogeneous_material_bit_exact():
    """per-element cohesion and friction angle (the config-3/5 material
    model) through a whole load-stepped solve"""
    n = 24
    w = ip.WellboreMesh(ip.wellbore_params(n, material_mode=2, c_cv=0.3, pw_final=-5.0))
    sm = ip.ElastoPlasticIntPointsStructMatrix(w)
    P = po.OracleProblem(po.default_params(n, material_mode=2, c_cv=0.3, pw_final=-5.0), nthreads=0)
    ug, uo = np.zeros(sm.neq), np.zeros(sm.neq)
    sg, lg = sm.newton(ug, 6, newton_max_it=25)
    so, lo = P.solve_steps(uo, 6, newton_max_it=25)
    assert sg.newton_iters == so.newton_iters and _eq(lg, lo) and _eq(ug, uo)
    assert np.array_equal(sm.get_state(3), P.arr("mtype").astype(np.float64))


def test_single_element_mesh():
    w = ip.WellboreMesh(ip.wellbore_params(1))
    sm = ip.ElastoPlasticIntPointsStructMatrix(w)
    P = po.OracleProblem(po.default_params(1), nthreads=0)
    assert sm.n_colors == 1
    ug, uo = np.zeros(sm.neq), np.zeros(sm.neq)
    sm.newton(ug, 2)
    P.solve_steps(uo, 2)
    assert _eq(ug, uo)


def test_nan_is_reported():
    w = ip.WellboreMesh(ip.wellbore_params(6))
    sm = ip.ElastoPlasticIntPointsStructMatrix(w)
    u = np.zeros(sm.neq)
    u[7] = np.nan
    r = sm.assemble_residual(u, np.zeros(sm.neq))
    assert np.isnan(r).any()
    sm.assemble(np.zeros(sm.neq), np.zeros(sm.neq))
    b = np.zeros(sm.neq)
    b[5] = np.nan
    with pytest.raises(ip.IpfemError) as e:
        sm.solve(b)
    assert e.value.status in (2, 3)


def test_cg_iteration_limit_and_state_roundtrip():
    w = ip.WellboreMesh(ip.wellbore_params(12))
    sm = ip.ElastoPlasticIntPointsStructMatrix(w)
    sm.SetLoadFactor(0.5)
    r = sm.assemble(np.zeros(sm.neq), np.zeros(sm.neq))
    with pytest.raises(ip.IpfemError) as e:
        sm.solve(r, max_it=3)
    assert e.value.status == 1
    x, it = sm.solve(r, max_it=3, allow_nonconverged=True)
    assert it == 3
    s0 = sm.get_state(0)
    s0[::7] += 1e-4
    sm.set_state(0, s0)
    assert np.array_equal(sm.get_state(0), s0)


def test_invalid_meshes_are_rejected():
    w = ip.WellboreMesh(ip.wellbore_params(3))
    con = w.array("connects").copy()
    con[4] = con[0]                           # repeated connect in an element
    m = ip.Mesh()
    C.memmove(C.byref(m), C.byref(w.mesh), C.sizeof(ip.Mesh))
    m.connects = con.ctypes.data_as(C.POINTER(C.c_int32))
    with pytest.raises(ip.IpfemError) as e:
        ip.ElastoPlasticIntPointsStructMatrix(m, w.material, keep=(w, con))
    assert e.value.status == 5
    con2 = w.array("connects").copy()
    con2[0] = 10 ** 6                          # connect out of range
    m.connects = con2.ctypes.data_as(C.POINTER(C.c_int32))
    with pytest.raises(ip.IpfemError):
        ip.ElastoPlasticIntPointsStructMatrix(m, w.material, keep=(w, con2))
    m.n_elements = 0
    with pytest.raises(ip.IpfemError):
        ip.ElastoPlasticIntPointsStructMatrix(m, w.material, keep=(w, con2))


def test_device_pointer_kernels_match_oracle():
    """TPZCudaCalls-level entry points on device buffers: Multiply
    (gather + B u), ComputeSigma, MultiplyTranspose"""
    n = 12
    w = ip.WellboreMesh(ip.wellbore_params(n))
    sm = ip.ElastoPlasticIntPointsStructMatrix(w)
    P = po.OracleProblem(po.default_params(n), nthreads=0)
    rng = np.random.default_rng(4)
    u = rng.normal(size=sm.neq) * 3e-3
    du = torch.tensor(u, device="cuda")
    st = torch.zeros(3 * sm.n_ip, dtype=torch.float64, device="cuda")
    sw = torch.zeros_like(st)
    res = torch.zeros(sm.neq, dtype=torch.float64, device="cuda")
    sm.gather_strain(du, st)
    P.assemble_residual(u.copy(), 0.0)          # fills the oracle's strain and sigma_w
    assert _eq(st.cpu().numpy().reshape(3, -1).T.ravel(), P.arr("strain"))
    sm.compute_sigma(0, st, sw)
    assert _eq(sw.cpu().numpy().reshape(3, -1).T.ravel(), P.arr("sigma_w"))
    sm.scatter_residual(sw, res)
    scat = np.zeros(P.neq)
    po.lib().orc_scatter_residual(P._p, po.ptr(P.arr("sigma_w")), po.ptr(scat))
    assert _eq(res.cpu().numpy(), scat)


def test_iteration_log_records_every_newton_iteration(tmp_path):
    """ipfem_set_iteration_log: one JSON line per Newton iteration (its CG
    count and |R| equal the solve's own log) and one per accepted load step"""
    import json

    sm, _ = (ip.ElastoPlasticIntPointsStructMatrix(ip.WellboreMesh(ip.wellbore_params(8))), None)
    path = str(tmp_path / "newton.jsonl")
    sm.set_iteration_log(path)
    u = np.zeros(sm.neq)
    st, log = sm.newton(u, 10, 0, 3, newton_max_it=30)
    sm.set_iteration_log(None)
    recs = [json.loads(line) for line in open(path)]
    its = [r for r in recs if "iter" in r]
    acc = [r for r in recs if r.get("accepted")]
    assert len(its) == st.newton_iters and len(acc) == 3
    assert [r["cg_iters"] for r in its] == log[:, 1].astype(int).tolist()
    assert [r["res"] for r in its] == log[:, 2].tolist()
    assert all(r["converged"] and r["res_rel"] <= 1e-8 for r in acc)
    assert all(r["ms_solve"] > 0 and r["ips_assemble"] > 0 for r in its)
    # closing the log stops the records
    sm.newton(np.zeros(sm.neq), 10, 0, 1, newton_max_it=30)
    assert len(open(path).readlines()) == len(recs)


def test_checkpoint_resume_is_bit_identical(tmp_path):
    """save u and the integration-point state after load step 3, restore them
    into a new context and continue: steps 4-6 give the iterates and state of
    the uninterrupted solve bit for bit"""
    w = ip.WellboreMesh(ip.wellbore_params(12, material_mode=2))
    a = ip.ElastoPlasticIntPointsStructMatrix(w)
    ua = np.zeros(a.neq)
    a.newton(ua, 10, 0, 3, newton_max_it=30)
    path = str(tmp_path / "step3.npz")
    a.save_checkpoint(path, ua, 3)
    a.newton(ua, 10, 3, 6, newton_max_it=30)
    b = ip.ElastoPlasticIntPointsStructMatrix(w)
    ub, step = b.load_checkpoint(path)
    assert step == 3
    b.newton(ub, 10, step, 6, newton_max_it=30)
    assert _eq(ua, ub)
    for f in range(4):
        assert _eq(a.get_state(f), b.get_state(f)), f
