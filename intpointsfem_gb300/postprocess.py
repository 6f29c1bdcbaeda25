"""Post-processing of a solution: the fields the reference writes and its line probes.

The reference's PostProcess (main.cpp:289-324) writes the integration-point
variables FailureType, Displacement, Stress, Strain and StrainPlastic through
NeoPZ's L2 projection onto a graphical mesh (TPZPostProcAnalysis::TransferSolution)
into a VTK file; its verification data are line probes of that file
(mathematica_notebooks/RK_Verification/*.csv, ParaView's column names).

Here, on the host with numpy (post-processing is not on the solver's path):
  - integration-point fields from the solution: total strain B u (tensor
    components, epsilon_xy = gamma_xy / 2, epsilon_zz = 0 in plane strain),
    the committed stress and plastic strain, m_type as the failure type;
  - an L2 projection of every field onto each element's Lagrange space,
    averaged at the shared connects weighted by element area;
  - point evaluation on the finite-element space (the displacement itself,
    the projected fields), with the bilinear geometry inverted by Newton;
  - line probes as CSV with the reference's columns, and a legacy VTK file
    (VTK_QUAD, VTK_BIQUADRATIC_QUAD or VTK_LAGRANGE_QUADRILATERAL by order;
    triangles of mixed meshes as VTK_TRIANGLE, VTK_QUADRATIC_TRIANGLE or
    VTK_LAGRANGE_TRIANGLE, their ghost connects left out).
Tensors are written as 3x3 row-major (xx, xy, xz, yx, yy, yz, zx, zy, zz).
"""
import numpy as np

COLUMNS = (["FailureType"] + ["Displacement:%d" % i for i in range(3)] + ["Stress:%d" % i for i in range(9)] +
           ["Strain:%d" % i for i in range(9)] + ["StrainPlastic:%d" % i for i in range(9)] +
           ["vtkValidPointMask", "arc_length", "Points:0", "Points:1", "Points:2"])


def ref_nodes(p):
    """index-space positions (a, b) in [0, p]^2 of the connects of an order-p
    element, in the library's connect order: vertices, the p-1 nodes of each
    edge in traversal order (v0v1, v1v2, v2v3, v3v0), interior row by row"""
    out = [(0, 0), (p, 0), (p, p), (0, p)]
    for e in range(4):
        for k in range(1, p):
            out.append([(k, 0), (p, k), (p - k, p), (0, p - k)][e])
    for b in range(1, p):
        for a in range(1, p):
            out.append((a, b))
    return out


def lagrange_1d(p, x):
    """[p+1, len(x)] values of the 1-D Lagrange functions on -1 + 2m/p"""
    x = np.asarray(x, dtype=np.float64)
    t = -1.0 + 2.0 * np.arange(p + 1) / p
    L = np.ones((p + 1,) + x.shape)
    for a in range(p + 1):
        for m in range(p + 1):
            if m != a:
                L[a] = L[a] * (x - t[m]) / (t[a] - t[m])
    return L


def shape(p, xi, eta):
    """[nn, len(xi)] tensor-product Lagrange functions of the connects"""
    lx, ly = lagrange_1d(p, xi), lagrange_1d(p, eta)
    return np.stack([lx[a] * ly[b] for a, b in ref_nodes(p)])


def gauss(p):
    x, w = np.polynomial.legendre.leggauss(p + 1)
    return x, w


def tri_nodes(p):
    """barycentric indices (i, j, k) of the connects of an order-p triangle, in the
    library's order: vertices, the p-1 nodes of each edge in traversal order
    (v0v1, v1v2, v2v0), the interior node (p = 3)"""
    out = [(p, 0, 0), (0, p, 0), (0, 0, p)]
    for e in range(3):
        for m in range(1, p):
            out.append([(p - m, m, 0), (0, p - m, m), (m, 0, p - m)][e])
    if p == 3:
        out.append((1, 1, 1))
    return out


def tri_shape(p, xi, eta, nn):
    """[nn, len(xi)] Lagrange functions of an order-p triangle at (xi, eta) of the
    unit triangle, zero rows for the ghost connects up to nn"""
    xi, eta = np.asarray(xi, dtype=np.float64), np.asarray(eta, dtype=np.float64)
    L = (1.0 - xi - eta, xi, eta)
    out = np.zeros((nn,) + xi.shape)
    for n, b in enumerate(tri_nodes(p)):
        v = np.ones_like(xi)
        for c in range(3):
            for s_ in range(b[c]):
                v = v * (p * L[c] - s_) / (s_ + 1)
        out[n] = v
    return out


def tri_points(p):
    """the collapsed Gauss points (xi, eta) of the library's order-p triangles"""
    gp, _ = gauss(p)
    n1 = p + 1
    u, v = 0.5 * (1 + np.tile(gp, n1)), 0.5 * (1 + np.repeat(gp, n1))
    return u, v * (1 - u)


class Solution:
    """A solution on a problem (WellboreMesh or GmshProblem): u [neq] and the
    committed state sigma [4][n_ip], eps_p [4][n_ip] (xx, xy, yy, zz), m_type [n_ip]."""

    def __init__(self, problem, u, sigma, eps_p, mtype):
        self.order = problem.order
        self.nn = (self.order + 1) ** 2
        self.con = problem.array("connects").reshape(-1, self.nn).astype(np.int64)
        sh = problem.array("el_shape")
        self.tri = np.zeros(len(self.con), bool) if sh is None else np.asarray(sh).astype(bool)
        self.nt = (self.order + 1) * (self.order + 2) // 2
        self.xy = problem.array("node_xy").reshape(-1, 2).copy()
        self.dphi = problem.array("dphi").reshape(-1, self.nn, 2, self.nn)
        self.weight = problem.array("weight").reshape(-1, self.nn)
        self.u = np.asarray(u, dtype=np.float64).reshape(-1, 2)
        n_ip = self.weight.size
        s, ep = np.asarray(sigma).reshape(4, n_ip), np.asarray(eps_p).reshape(4, n_ip)
        ue = self.u[self.con]                                     # [e, n, 2]
        exx = np.einsum("eqn,en->eq", self.dphi[:, :, 0, :], ue[:, :, 0]).ravel()
        eyy = np.einsum("eqn,en->eq", self.dphi[:, :, 1, :], ue[:, :, 1]).ravel()
        gxy = (np.einsum("eqn,en->eq", self.dphi[:, :, 1, :], ue[:, :, 0]) +
               np.einsum("eqn,en->eq", self.dphi[:, :, 0, :], ue[:, :, 1])).ravel()
        z = np.zeros(n_ip)

        def tensor(xx, xy, yy, zz):
            return np.stack([xx, xy, z, xy, yy, z, z, z, zz], 1)

        self.ip = {"FailureType": np.asarray(mtype, dtype=np.float64).reshape(n_ip, 1),
                   "Stress": tensor(s[0], s[1], s[2], s[3]),
                   "Strain": tensor(exx, 0.5 * gxy, eyy, z),
                   "StrainPlastic": tensor(ep[0], ep[1], ep[2], ep[3])}
        self._nodal = None

    @classmethod
    def from_struct_matrix(cls, problem, sm, u):
        return cls(problem, u, sm.get_state(1), sm.get_state(0), sm.get_state(3))

    def nodal(self):
        """L2 projection of the integration-point fields onto each element's
        Lagrange space (M_e c = b_e with M_e = sum_q w_q N N^T), averaged at the
        shared connects weighted by element area"""
        if self._nodal is None:
            gp, _ = gauss(self.order)
            n1 = self.order + 1
            Nq = shape(self.order, np.tile(gp, n1), np.repeat(gp, n1))     # [nn, q]
            Nt = tri_shape(self.order, *tri_points(self.order), self.nt)   # [nt, q]
            den = np.zeros(len(self.xy))
            num = {k: np.zeros((len(self.xy), f.shape[1])) for k, f in self.ip.items()}
            n_el = self.weight.shape[0]
            for mask, N in ((~self.tri, Nq), (self.tri, Nt)):
                if not mask.any():
                    continue
                n = N.shape[0]
                w = self.weight[mask]                                       # [E, q]
                M = np.einsum("nq,mq,eq->enm", N, N, w)
                area = w.sum(1)
                con = self.con[mask][:, :n]
                np.add.at(den, con, np.repeat(area[:, None], n, 1))
                for k, f in self.ip.items():
                    fq = f.reshape(n_el, self.nn, -1)[mask]                 # [E, q, c]
                    c = np.linalg.solve(M, np.einsum("nq,eq,eqc->enc", N, w, fq))
                    np.add.at(num[k], con, c * area[:, None, None])
            # ghost connects of triangles belong to no element's space: 0 there
            self._nodal = {k: np.divide(v, den[:, None], out=np.zeros_like(v), where=den[:, None] != 0)
                           for k, v in num.items()}
        return self._nodal

    def _inside(self, e, x, tol):
        """reference coordinates of x in element e, or None outside it"""
        v = self._V[e]
        if self.tri[e]:
            J = np.stack([v[1] - v[0], v[2] - v[0]], 1)
            s = np.linalg.solve(J, x - v[0])
            return s if (s.min() >= -tol and s.sum() <= 1 + tol) else None
        s = np.zeros(2)
        for _ in range(30):
            xi, et = s
            Nv = 0.25 * np.array([(1 - xi) * (1 - et), (1 + xi) * (1 - et), (1 + xi) * (1 + et),
                                  (1 - xi) * (1 + et)])
            dN = 0.25 * np.array([[-(1 - et), (1 - et), (1 + et), -(1 + et)],
                                  [-(1 - xi), -(1 + xi), (1 + xi), (1 - xi)]])
            r = Nv @ v - x
            J = dN @ v                                                     # [2 (xi, eta), 2 (x, y)]
            step = np.linalg.solve(J.T, r)
            s = s - step
            if np.abs(step).max() < 1e-14:
                break
        return np.clip(s, -1, 1) if np.all(np.abs(s) <= 1 + tol) else None

    def _index(self):
        """element vertices, bounding boxes and a uniform grid of cells, each
        listing (in ascending order) the elements whose bounding box overlaps it"""
        if getattr(self, "_V", None) is not None:
            return
        V = self.xy[self.con[:, :4]]                                       # [e, 4, 2]
        V[self.tri, 3] = V[self.tri, 2]                                    # triangles: 3 vertices
        self._V = V
        lo, hi = V.min(1) - 1e-12, V.max(1) + 1e-12
        self._lo, self._hi = lo, hi
        g = max(1, int(np.sqrt(len(V))))
        x0, x1 = lo.min(0), hi.max(0)
        h = np.where(x1 > x0, (x1 - x0) / g, 1.0)
        self._grid = (g, x0, h)
        i0 = np.clip(np.floor((lo - x0) / h).astype(np.int64), 0, g - 1)
        i1 = np.clip(np.floor((hi - x0) / h).astype(np.int64), 0, g - 1)
        nx, ny = i1[:, 0] - i0[:, 0] + 1, i1[:, 1] - i0[:, 1] + 1
        cnt = nx * ny
        el = np.repeat(np.arange(len(V)), cnt)                             # ascending element order
        k = np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt)    # index inside each element's block
        cx = i0[el, 0] + k % nx[el]
        cy = i0[el, 1] + k // nx[el]
        cell = cy * g + cx
        order = np.argsort(cell, kind="stable")                            # stable: elements stay ascending
        self._cell_el = el[order]
        self._cell_ptr = np.searchsorted(cell[order], np.arange(g * g + 1))

    def _candidates(self, x):
        """ascending elements whose bounding box contains x"""
        g, x0, h = self._grid
        c = np.floor((x - x0) / h).astype(np.int64)
        if np.any(c < 0) or np.any(c >= g):
            # outside the grid: only elements whose box reaches past it
            # (none, as the grid spans every box), so nothing contains x
            return np.zeros(0, np.int64)
        cid = c[1] * g + c[0]
        cand = self._cell_el[self._cell_ptr[cid]:self._cell_ptr[cid + 1]]
        return cand[np.all((x >= self._lo[cand]) & (x <= self._hi[cand]), 1)]

    def locate(self, pts, tol=1e-10, scan=False):
        """element and reference coordinates of each point (element -1 outside):
        the lowest-numbered element that contains it.  Every element whose
        bounding box contains the point is listed, in ascending order, in the
        grid cell of the point (the cells an element is filed under cover its
        box), so the grid path tests exactly the elements, in the same order,
        that the full scan (scan=True) tests, and picks the same element."""
        self._index()
        lo, hi = self._lo, self._hi
        pts = np.asarray(pts, dtype=np.float64).reshape(-1, 2)
        el = np.full(len(pts), -1)
        ref = np.zeros((len(pts), 2))
        for i, x in enumerate(pts):
            cand = np.nonzero(np.all((x >= lo) & (x <= hi), 1))[0] if scan else self._candidates(x)
            for e in cand:
                s = self._inside(e, x, tol)
                if s is not None:
                    el[i], ref[i] = e, s
                    break
        return el, ref

    def evaluate(self, pts):
        """dict of field values at the points (the displacement is the finite-
        element field itself; NaN outside the mesh) and the validity mask"""
        el, ref = self.locate(pts)
        ok = el >= 0
        N = shape(self.order, ref[:, 0], ref[:, 1]).T                      # [pts, n]
        on_tri = ok & self.tri[np.maximum(el, 0)]
        if on_tri.any():
            N[on_tri] = tri_shape(self.order, ref[on_tri, 0], ref[on_tri, 1], self.nn).T
        nodes = self.con[np.maximum(el, 0)]                                # [pts, n]
        out = {"Displacement": np.einsum("pn,pnc->pc", N, self.u[nodes])}
        for k, f in self.nodal().items():
            out[k] = np.einsum("pn,pnc->pc", N, f[nodes])
        for k in out:
            out[k][~ok] = np.nan
        return out, ok

    def line_probe(self, p0, p1, n_points=1001):
        """rows of the reference's CSV columns along the segment p0-p1"""
        p0, p1 = np.asarray(p0, dtype=np.float64), np.asarray(p1, dtype=np.float64)
        t = np.linspace(0.0, 1.0, n_points)
        pts = p0[None, :] + t[:, None] * (p1 - p0)[None, :]
        vals, ok = self.evaluate(pts)
        disp = np.concatenate([vals["Displacement"], np.zeros((n_points, 1))], 1)
        cols = [vals["FailureType"], disp, vals["Stress"], vals["Strain"], vals["StrainPlastic"],
                ok.astype(np.float64)[:, None], (t * np.linalg.norm(p1 - p0))[:, None], pts,
                np.zeros((n_points, 1))]
        return np.concatenate(cols, 1)

    def write_line_probe_csv(self, path, p0, p1, n_points=1001):
        rows = self.line_probe(p0, p1, n_points)
        with open(path, "w") as f:
            f.write(",".join('"%s"' % c for c in COLUMNS) + "\n")
            for r in rows:
                f.write(",".join("%.10g" % v for v in r) + "\n")
        return rows

    def write_vtk(self, path):
        """legacy ASCII VTK unstructured grid of the connects with the projected fields"""
        p = self.order
        cell_type = {1: 9, 2: 28, 3: 70}[p]
        tri_type = {1: 5, 2: 22, 3: 69}[p]                                 # triangles: ghosts left out
        perm = list(range(self.nn))
        if p == 3:
            # VTK runs edge 2 from v3 to v2 and edge 3 from v0 to v3
            e2, e3 = 4 + 2 * (p - 1), 4 + 3 * (p - 1)
            perm[e2:e2 + p - 1] = perm[e2:e2 + p - 1][::-1]
            perm[e3:e3 + p - 1] = perm[e3:e3 + p - 1][::-1]
        nodal = self.nodal()
        n_el, n_pt = self.con.shape[0], len(self.xy)
        cells = [self.con[e, :self.nt] if self.tri[e] else self.con[e, perm] for e in range(n_el)]
        n_ent = sum(len(c) + 1 for c in cells)
        with open(path, "w") as f:
            f.write("# vtk DataFile Version 3.0\nelastoplastic solution, order %d\nASCII\n"
                    "DATASET UNSTRUCTURED_GRID\n" % p)
            f.write("POINTS %d double\n" % n_pt)
            np.savetxt(f, np.concatenate([self.xy, np.zeros((n_pt, 1))], 1), fmt="%.15g")
            f.write("CELLS %d %d\n" % (n_el, n_ent))
            for c in cells:
                f.write("%d %s\n" % (len(c), " ".join(str(int(v)) for v in c)))
            f.write("CELL_TYPES %d\n" % n_el)
            np.savetxt(f, np.where(self.tri, tri_type, cell_type), fmt="%d")
            f.write("POINT_DATA %d\n" % n_pt)
            f.write("SCALARS FailureType double 1\nLOOKUP_TABLE default\n")
            np.savetxt(f, nodal["FailureType"][:, 0], fmt="%.10g")
            f.write("VECTORS Displacement double\n")
            np.savetxt(f, np.concatenate([self.u, np.zeros((n_pt, 1))], 1), fmt="%.10g")
            for k in ("Stress", "Strain", "StrainPlastic"):
                f.write("TENSORS %s double\n" % k)
                np.savetxt(f, nodal[k].reshape(-1, 3), fmt="%.10g")
