"""Post-processing (the reference's PostProcess, main.cpp:289-324, and the line
probes of its verification data): projection, point evaluation, the CSV
columns of mathematica_notebooks/RK_Verification/*.csv and the VTK file, on
fields with known values."""
import os

import numpy as np
import pytest

ip = pytest.importorskip("intpointsfem_gb300")
from intpointsfem_gb300 import gmsh_wellbore as gw  # noqa: E402
from intpointsfem_gb300 import postprocess as pp  # noqa: E402

from oracle.build import reference_dir  # noqa: E402

REF_CSV = os.path.join(reference_dir(), "mathematica_notebooks", "RK_Verification", "ElastoPlasticFEMdata.csv")


def _problem(tmp_path, order, n=12, q=1.3):
    path = str(tmp_path / "wb.msh")
    gw.write_wellbore_msh(path, n, q)
    bcs, mat = gw.reference_bcs()
    return ip.GmshProblem(ip.GmshMesh(path), bcs, order=order, **mat)


@pytest.mark.parametrize("order", [1, 2, 3])
def test_probe_reproduces_linear_fields(tmp_path, order):
    """a linear displacement is reproduced exactly along a probe, its strain
    (tensor components, xy = gamma/2) and a constant stress are projected
    exactly; points in the hole are masked"""
    pb = _problem(tmp_path, order)
    xy = pb.array("node_xy").reshape(-1, 2)
    u = np.stack([1e-3 * xy[:, 0] + 2e-3 * xy[:, 1], -0.5e-3 * xy[:, 0] + 3e-3 * xy[:, 1]], 1).ravel()
    n_ip = pb.array("weight").size
    sig = np.tile(np.array([-1.0, 0.5, -2.0, -0.6])[:, None], (1, n_ip))
    ep = np.tile(np.array([1e-4, -2e-5, -1e-4, 0.0])[:, None], (1, n_ip))
    S = pp.Solution(pb, u, sig, ep, np.ones(n_ip))
    rows = S.write_line_probe_csv(str(tmp_path / "p.csv"), (0.1, 0.0), (3.0, 2.0), 101)
    c = {k: i for i, k in enumerate(pp.COLUMNS)}
    X, Y = rows[:, c["Points:0"]], rows[:, c["Points:1"]]
    assert rows[:, c["vtkValidPointMask"]].min() == 1.0
    assert np.abs(rows[:, c["Displacement:0"]] - (1e-3 * X + 2e-3 * Y)).max() < 1e-15
    assert np.abs(rows[:, c["Displacement:1"]] - (-0.5e-3 * X + 3e-3 * Y)).max() < 1e-15
    for col, v in (("Strain:0", 1e-3), ("Strain:1", 0.75e-3), ("Strain:3", 0.75e-3), ("Strain:4", 3e-3),
                   ("Strain:8", 0.0), ("Stress:0", -1.0), ("Stress:1", 0.5), ("Stress:4", -2.0), ("Stress:8", -0.6),
                   ("StrainPlastic:1", -2e-5), ("FailureType", 1.0)):
        assert np.abs(rows[:, c[col]] - v).max() < 1e-12 * max(1.0, abs(v)) + 1e-15, col
    assert abs(rows[-1, c["arc_length"]] - np.hypot(2.9, 2.0)) < 1e-12
    vals, ok = S.evaluate(np.array([[0.0, 0.0], [0.05, 0.0]]))
    assert not ok.any() and np.isnan(vals["Displacement"]).all()


def test_csv_header_is_the_reference_header(tmp_path):
    if not os.path.exists(REF_CSV):
        pytest.skip("reference CSV not present")
    with open(REF_CSV) as f:
        ref = [h.strip().strip('"') for h in f.readline().split(",")]
    assert ref == pp.COLUMNS


@pytest.mark.parametrize("order", [1, 2, 3])
def test_vtk_file(tmp_path, order):
    pb = _problem(tmp_path, order, n=6)
    n_ip = pb.array("weight").size
    S = pp.Solution(pb, np.zeros(pb.neq), np.zeros((4, n_ip)), np.zeros((4, n_ip)), np.zeros(n_ip))
    path = str(tmp_path / "s.vtk")
    S.write_vtk(path)
    lines = open(path).read().split("\n")
    nn = (order + 1) ** 2
    i = lines.index("POINTS %d double" % pb.n_nodes)
    j = lines.index("CELLS %d %d" % (pb.n_el, pb.n_el * (nn + 1)))
    k = lines.index("CELL_TYPES %d" % pb.n_el)
    assert j - i - 1 == pb.n_nodes and k - j - 1 == pb.n_el
    assert set(lines[k + 1:k + 1 + pb.n_el]) == {str({1: 9, 2: 28, 3: 70}[order])}
    cells = np.array([list(map(int, l.split())) for l in lines[j + 1:k]])
    assert (cells[:, 0] == nn).all() and set(np.unique(cells[:, 1:])) == set(range(pb.n_nodes))
    for name in ("SCALARS FailureType double 1", "VECTORS Displacement double", "TENSORS Stress double",
                 "TENSORS Strain double", "TENSORS StrainPlastic double"):
        assert name in lines


@pytest.mark.parametrize("order", [1, 2, 3])
def test_mixed_mesh_probe_and_vtk(tmp_path, order):
    """the same checks on a mixed triangle/quadrilateral mesh: a linear field
    and constant state reproduced along a probe that crosses both kinds of
    element, triangle cells in the VTK file without their ghost connects"""
    path = str(tmp_path / "mix.msh")
    gw.write_wellbore_msh(path, 9, 1.3, tri_quadrants=(1, 3))
    bcs, mat = gw.reference_bcs()
    pb = ip.GmshProblem(ip.GmshMesh(path), bcs, order=order, **mat)
    xy = pb.array("node_xy").reshape(-1, 2)
    u = np.stack([1e-3 * xy[:, 0] + 2e-3 * xy[:, 1], -0.5e-3 * xy[:, 0] + 3e-3 * xy[:, 1]], 1).ravel()
    n_ip = pb.array("weight").size
    sig = np.tile(np.array([-1.0, 0.5, -2.0, -0.6])[:, None], (1, n_ip))
    S = pp.Solution(pb, u, sig, np.zeros((4, n_ip)), np.ones(n_ip))
    rows = S.line_probe((2.0, 0.5), (-2.0, 1.0), 81)                  # quadrant 0 -> quadrant 1 (triangles)
    c = {k: i for i, k in enumerate(pp.COLUMNS)}
    X, Y = rows[:, c["Points:0"]], rows[:, c["Points:1"]]
    assert rows[:, c["vtkValidPointMask"]].min() == 1.0
    assert np.abs(rows[:, c["Displacement:0"]] - (1e-3 * X + 2e-3 * Y)).max() < 1e-15
    assert np.abs(rows[:, c["Strain:1"]] - 0.75e-3).max() < 1e-12
    assert np.abs(rows[:, c["Stress:4"]] + 2.0).max() < 1e-12
    S.write_vtk(str(tmp_path / "m.vtk"))
    lines = open(tmp_path / "m.vtk").read().split("\n")
    k = lines.index("CELL_TYPES %d" % pb.n_el)
    types = np.array(lines[k + 1:k + 1 + pb.n_el], dtype=int)
    assert (types == {1: 5, 2: 22, 3: 69}[order]).sum() == pb.array("el_shape").sum()


@pytest.mark.parametrize("tri", [(), (1, 3)])
@pytest.mark.parametrize("order", [1, 2])
def test_locate_grid_equals_full_scan(tmp_path, tri, order):
    """point location through the grid of element boxes picks the same element
    as the full scan over all elements, also for points exactly on element
    vertices and edges (several elements contain them: the lowest-numbered
    one is taken), on a graded quadrilateral mesh and on a mixed
    triangle/quadrilateral mesh, plus random points inside and outside"""
    path = str(tmp_path / "m.msh")
    gw.write_wellbore_msh(path, 9, 1.3, tri_quadrants=tri)
    bcs, mat = gw.reference_bcs()
    pb = ip.GmshProblem(ip.GmshMesh(path), bcs, order=order, **mat)
    n_ip = pb.array("weight").size
    z4 = np.zeros((4, n_ip))
    S = pp.Solution(pb, np.zeros(pb.neq), z4, z4, np.zeros(n_ip))
    S._index()
    V = S._V
    rng = np.random.default_rng(3)
    verts = V.reshape(-1, 2)
    mids = 0.5 * (V + np.roll(V, -1, axis=1)).reshape(-1, 2)               # edge midpoints
    lo, hi = verts.min(0), verts.max(0)
    rnd = lo + (hi - lo) * rng.random((400, 2))                            # the hole and beyond: some outside
    pts = np.concatenate([verts[rng.choice(len(verts), 300)], mids[rng.choice(len(mids), 300)], rnd])
    e_grid, r_grid = S.locate(pts)
    e_scan, r_scan = S.locate(pts, scan=True)
    assert np.array_equal(e_grid, e_scan)
    assert np.array_equal(r_grid, r_scan)
    assert (e_grid >= 0).sum() > 600 and (e_grid < 0).any()
