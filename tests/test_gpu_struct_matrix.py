"""The C++ struct-matrix class (include/ipfem_pz.hpp) on the GPU against the
oracle: a compiled C++ program drives Assemble(rhs), CreateAssemble(rhs),
Clone() and a state commit exactly as the reference's analysis drives
TPZElastoPlasticIntPointsStructMatrix; its residuals and its symmetric-upper
CSR tangent (TPZSYsmpMatrix's IA, JA, A) equal the oracle's bit for bit."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ip = pytest.importorskip("intpointsfem_gb300")
from oracle import pyoracle as po  # noqa: E402
from struct_matrix_build import build_driver  # noqa: E402


def sym_upper_csr(row_ptr, col, K, n_nodes):
    """nodal 2x2 blocks -> upper triangle of the dof matrix in CSR (rows and
    columns ascending), the storage of NeoPZ's TPZSYsmpMatrix"""
    ia, ja, a = [0], [], []
    K = K.reshape(-1, 2, 2)
    for i in range(n_nodes):
        for p in range(2):
            row = 2 * i + p
            for k in range(row_ptr[i], row_ptr[i + 1]):
                j = col[k]
                for q in range(2):
                    if 2 * j + q >= row:
                        ja.append(2 * j + q)
                        a.append(K[k, p, q])
            ia.append(len(ja))
    return np.array(ia), np.array(ja), np.array(a)


def _read(d, name, dtype=np.float64):
    return np.fromfile(os.path.join(d, name), dtype=dtype)


def test_struct_matrix_class_equals_oracle(tmp_path):
    n, lam = 12, 0.6
    exe = build_driver(tmp_path)
    P = po.OracleProblem(po.default_params(n, material_mode=0), nthreads=0)
    rng = np.random.default_rng(4)
    u = rng.normal(size=P.neq) * 2e-3
    u[P.arr("fixed").astype(bool)] = 0.0
    u.tofile(str(tmp_path / "u.bin"))
    r = subprocess.run([exe, str(n), str(lam), str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.stdout, r.stderr)
    assert "error path: ipfem: invalid argument: load factor is not finite" in r.stdout
    d = str(tmp_path)
    # Assemble(rhs)
    assert np.array_equal(_read(d, "res.bin"), P.assemble_residual(u.copy(), lam))
    # CreateAssemble(rhs): residual and tangent in TPZSYsmpMatrix form
    assert np.array_equal(_read(d, "rhs_k.bin"), P.assemble(u.copy(), lam))
    ia, ja, a = sym_upper_csr(P.arr("row_ptr"), P.arr("col"), P.arr("K"), P.n_nodes)
    assert np.array_equal(_read(d, "ia.bin", np.int64), ia)
    assert np.array_equal(_read(d, "ja.bin", np.int64), ja)
    assert np.array_equal(_read(d, "pattern_ja.bin", np.int64), ja)
    assert np.array_equal(_read(d, "a.bin"), a)
    # the clone evaluates the same residual
    assert np.array_equal(_read(d, "clone_res.bin"), _read(d, "res.bin"))
    # state commit through SetUpdateMem, then the next residual. This random u
    # drives some points to the apex; evaluated again at the same strain, such a
    # point has zero elastic strain, and the reference's spectral decomposition
    # (FunctionsStressStrain.h, ComputeSigma) returns NaN there. The library and
    # the oracle give NaN at the same entries and equal bits elsewhere.
    P.assemble_residual(u.copy(), lam, update_mem=True)
    after, want = _read(d, "res_after_commit.bin"), P.assemble_residual(u.copy(), lam)
    assert np.array_equal(np.isnan(after), np.isnan(want))
    assert np.array_equal(after, want, equal_nan=True)


def test_sym_csr_export_matches_blocks():
    """ipfem_get_stiffness_sym_csr against the block export of the same
    tangent, mixed precision included"""
    w = ip.WellboreMesh(ip.wellbore_params(10, material_mode=2))
    sm = ip.ElastoPlasticIntPointsStructMatrix(w)
    rng = np.random.default_rng(9)
    u = rng.normal(size=sm.neq) * 1e-3
    for mode in (ip.PLAIN_FP64, ip.MIXED):
        sm.set_precision(mode)
        sm.SetLoadFactor(1.0)
        sm.assemble(u, np.zeros(sm.neq))
        rp, col, K = sm.stiffness()
        ia, ja, a = sm.stiffness_sym_csr()
        ia2, ja2, a2 = sym_upper_csr(rp, col, K, sm.n_nodes)
        assert np.array_equal(ia, ia2) and np.array_equal(ja, ja2) and np.array_equal(a, a2)
        assert a.size == 4 * (rp[-1] - sm.n_nodes) // 2 + 3 * sm.n_nodes
