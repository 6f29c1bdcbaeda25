"""GB300-native integration-point FEM: Python view of libipfem's C-ABI.

The compute path is libipfem.so (hand-written sm_103a CUDA behind the C-ABI
of include/ipfem.h).  This module only binds it with ctypes and mirrors the
reference's TPZElastoPlasticIntPointsStructMatrix interface
(TPZElastoPlasticIntPointsStructMatrix.h:33-42) so that tests and benchmarks
read like the reference's own calls.  There is no CPU fallback: if the
library or a device is missing, every entry point raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libipfem.so")

HOST, DEVICE = 0, 1
PLAIN_FP64, MIXED = 0, 1
PREC_JACOBI, PREC_MLP, PREC_BLOCK_JACOBI = 0, 1, 2
MLP_PARAMS = 23316
# Inner (FP32 flexible-CG) tolerance of the chosen method, mixed precision +
# learned preconditioner, inside the FP64 Newton loop to 1e-8: the adaptive
# forcing term (ipfem_set_inner_tolerance) with the first solve of each load
# step to CHOSEN_CG_RTOL.  Measured over the whole 20-step 400 x 400 solve on a
# GB300: fixed tolerances 1e-2: 24.3 s (163 Newton iterations), 3e-3: 18.9 s
# (148), 1e-3: 22.1 s (148), 1e-4: 30.2 s (148); adaptive (gamma 0.9, alpha 2,
# eta in [1e-4, 0.3], first solve 3e-2): 16.0 s (151 Newton iterations, 17 %
# fewer CG iterations), u and sigma within 3e-10 of the fixed-3e-3 solve.
CHOSEN_CG_RTOL = 3e-2
CHOSEN_INNER = dict(mode=1, gamma=0.9, alpha=2.0, eta_min=1e-4, eta_max=0.3)
FIXED_CG_RTOL = 3e-3       # the best fixed inner tolerance (mode 0)
# The chosen method also starts each load step from the secant prediction
# (ipfem_set_newton_predictor): the same 400 x 400 solve in 6.2 s (98 Newton,
# 64 248 CG iterations) instead of 15.1 s, the elastic steps converging in one
# Newton iteration from a start at ~1e-7 of their residual.
CHOSEN_PREDICTOR = True
# ... and assembles the consistent spectral tangent (ipfem_set_consistent_tangent):
# 400 x 400 in 4.95 s (51 Newton, 52 816 CG iterations) instead of 6.41 s (95,
# 67 547), u within 8e-11 and sigma within 1.5e-10 of the solve with the
# reference's tangent.  The plain FP64 method keeps the reference's tangent.
CHOSEN_CONSISTENT_TANGENT = True


def use_chosen_newton(sm):
    """the chosen method's Newton settings on a struct matrix in IPFEM_MIXED:
    adaptive inner tolerance (pass CHOSEN_CG_RTOL as cg_rtol), the secant
    predictor and the consistent tangent"""
    sm.set_inner_tolerance(**CHOSEN_INNER)
    sm.set_newton_predictor(CHOSEN_PREDICTOR)
    sm.set_consistent_tangent(CHOSEN_CONSISTENT_TANGENT)


STATUS = {0: "ok", 1: "not converged", 2: "non-finite value", 3: "CG breakdown", 4: "out of device memory",
          5: "invalid argument", 6: "CUDA error", 7: "no sm_103 device"}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_lp = C.POINTER(C.c_int64)
_bp = C.POINTER(C.c_uint8)


class IpfemError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("ipfem: %s (%d): %s" % (STATUS.get(status, "?"), status, msg))
        self.status = status


class Mesh(C.Structure):
    _fields_ = [("n_elements", C.c_int32), ("n_nodes", C.c_int32), ("connects", _ip), ("dphi", _dp),
                ("block_storage", _dp), ("weight", _dp), ("fixed", _bp), ("f0", _dp), ("df", _dp),
                ("order", C.c_int32)]


class Material(C.Structure):
    _fields_ = [("E", C.c_double), ("nu", C.c_double), ("cohesion", C.c_double), ("phi", C.c_double),
                ("psi", C.c_double), ("el_cohesion", _dp), ("el_phi", _dp), ("sigma0", C.c_double * 4)]


class SolveOpts(C.Structure):
    _fields_ = [("n_steps", C.c_int32), ("newton_rtol", C.c_double), ("newton_max_it", C.c_int32),
                ("cg_rtol", C.c_double), ("cg_max_it", C.c_int32)]


class SolveStats(C.Structure):
    _fields_ = [("newton_iters", C.c_int32), ("cg_iters", C.c_int64), ("last_step_iters", C.c_int32),
                ("converged", C.c_int32), ("final_res", C.c_double), ("ms_assemble", C.c_double),
                ("ms_solve", C.c_double), ("ms_commit", C.c_double), ("fcg_fallbacks", C.c_int64)]


class WellboreParams(C.Structure):
    _fields_ = [("nr", C.c_int32), ("nt", C.c_int32), ("r_in", C.c_double), ("r_out", C.c_double),
                ("grading", C.c_double), ("E", C.c_double), ("nu", C.c_double), ("cohesion", C.c_double),
                ("phi_deg", C.c_double), ("psi_deg", C.c_double), ("sxx0", C.c_double), ("syy0", C.c_double),
                ("sxy0", C.c_double), ("szz0", C.c_double), ("pw_final", C.c_double),
                ("material_mode", C.c_int32), ("c_cv", C.c_double), ("phi_lo_deg", C.c_double),
                ("phi_hi_deg", C.c_double), ("seed", C.c_uint64)]


class Wellbore(C.Structure):
    _fields_ = [("mesh", Mesh), ("material", Material), ("node_xy", _dp), ("connects", _ip), ("dphi", _dp),
                ("weight", _dp), ("f0", _dp), ("df", _dp), ("el_cohesion", _dp), ("el_phi", _dp),
                ("fixed", _bp), ("el_shape", _bp), ("n_ghost", C.c_int32)]


class GmshData(C.Structure):
    _fields_ = [("n_nodes", C.c_int32), ("xy", _dp), ("n_quads", C.c_int32), ("quads", _ip), ("quad_phys", _ip),
                ("n_lines", C.c_int32), ("lines", _ip), ("line_phys", _ip), ("n_points", C.c_int32),
                ("points", _ip), ("point_phys", _ip), ("n_phys", C.c_int32), ("phys_dim", _ip),
                ("phys_tag", _ip), ("phys_name", C.POINTER(C.c_char_p)), ("n_tris", C.c_int32), ("tris", _ip),
                ("tri_phys", _ip)]


class BC(C.Structure):
    _fields_ = [("phys", C.c_int32), ("type", C.c_int32), ("val", C.c_double * 2)]


_lib = None


def lib():
    """Load libipfem.so (in-tree build); raises if it is not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libipfem.so is not built; run intpointsfem_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        S = C.c_int
        P = C.c_void_p
        sig = {
            "ipfem_create": (S, [C.POINTER(Mesh), C.POINTER(Material), C.POINTER(P)]),
            "ipfem_destroy": (None, [P]),
            "ipfem_last_error": (C.c_char_p, [P]),
            "ipfem_status_string": (C.c_char_p, [S]),
            "ipfem_sizes": (S, [P, _lp]),
            "ipfem_stream": (P, [P]),
            "ipfem_set_load_factor": (S, [P, C.c_double]),
            "ipfem_set_update_mem": (S, [P, S]),
            "ipfem_set_precision": (S, [P, S]),
            "ipfem_set_residual_precision": (S, [P, S, C.c_double]),
            "ipfem_assemble_residual": (S, [P, P, P, S]),
            "ipfem_assemble": (S, [P, P, P, S]),
            "ipfem_get_stiffness": (S, [P, _lp, _ip, _dp]),
            "ipfem_get_stiffness_sym_csr": (S, [P, _lp, _lp, _lp, _dp]),
            "ipfem_solve": (S, [P, P, P, C.c_double, S, S, C.POINTER(C.c_int)]),
            "ipfem_newton_solve": (S, [P, C.POINTER(SolveOpts), C.c_int32, C.c_int32, P, S,
                                       C.POINTER(SolveStats), _dp, C.c_int32]),
            "ipfem_newton_begin": (S, [P, C.POINTER(SolveOpts), C.c_int32, C.c_int32]),
            "ipfem_set_newton_accel": (S, [P, S]),
            "ipfem_newton_advance": (S, [P, C.c_int32, P, S, C.POINTER(SolveStats), _dp, C.c_int32,
                                         C.POINTER(C.c_int32)]),
            "ipfem_dot": (S, [P, P, P, _dp]),
            "ipfem_dot_noalloc": (S, [P, P, C.c_int64, P, P]),
            "ipfem_launch_count": (C.c_uint64, [P]),
            "ipfem_set_iteration_log": (S, [P, C.c_char_p]),
            "ipfem_profile_spmv": (S, [P, S, _dp]),
            "ipfem_profile_residual": (S, [P, P, S, S, _dp]),
            "ipfem_measure_fp64_peak": (S, [P, _dp]),
            "ipfem_set_node_grid": (S, [P, C.c_int32, C.c_int32]),
            "ipfem_mlp_init": (S, [P, C.c_uint64]),
            "ipfem_set_preconditioner": (S, [P, S]),
            "ipfem_mlp_get_params": (S, [P, C.POINTER(C.c_float)]),
            "ipfem_mlp_set_params": (S, [P, C.POINTER(C.c_float)]),
            "ipfem_mlp_features": (S, [P, P]),
            "ipfem_mlp_forward": (S, [P, P, C.c_int64, P]),
            "ipfem_mlp_operator": (S, [P, P]),
            "ipfem_learn_grad": (S, [P, P, P, S, C.c_float, C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
            "ipfem_mlp_adam": (S, [P, C.POINTER(C.c_float), C.c_float]),
            "ipfem_cg_snapshots": (S, [P, P, C.c_double, S, S, _ip, P, P, P, C.POINTER(C.c_int)]),
            "ipfem_gather_strain": (S, [P, P, P]),
            "ipfem_compute_sigma": (S, [P, S, P, P, P]),
            "ipfem_scatter_residual": (S, [P, P, P]),
            "ipfem_gather_strain32": (S, [P, P, P]),
            "ipfem_scatter_residual32": (S, [P, P, P]),
            "ipfem_get_state": (S, [P, S, _dp]),
            "ipfem_set_state": (S, [P, S, _dp]),
            "ipfem_get_setup": (S, [P, S, P]),
            "ipfem_color_elements": (C.c_int32, [C.c_int32, C.c_int32, _ip, _ip]),
            "ipfem_color_elements_nn": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, _ip, _ip]),
            "ipfem_wellbore_default": (None, [C.POINTER(WellboreParams), C.c_int32]),
            "ipfem_wellbore_build": (S, [C.POINTER(WellboreParams), C.POINTER(C.POINTER(Wellbore))]),
            "ipfem_wellbore_free": (None, [C.POINTER(Wellbore)]),
            "ipfem_set_newton_tangent": (S, [P, S]),
            "ipfem_set_inner_tolerance": (S, [P, S, C.c_double, C.c_double, C.c_double, C.c_double]),
            "ipfem_set_newton_predictor": (S, [P, S]),
            "ipfem_set_consistent_tangent": (S, [P, S]),
            "ipfem_set_spectral_mode": (S, [P, S]),
            "ipfem_set_row_stencils": (S, [P, S]),
            "ipfem_row_stencil_count": (S, [P, _ip, _ip]),
            "ipfem_layout_info": (S, [P, S, _lp, _lp, _ip]),
            "ipfem_gmsh_read": (S, [C.c_char_p, C.POINTER(C.POINTER(GmshData))]),
            "ipfem_gmsh_free": (None, [C.POINTER(GmshData)]),
            "ipfem_gmsh_problem": (S, [C.POINTER(GmshData), C.c_int32, C.c_int32, C.POINTER(BC), C.c_int32,
                                       C.POINTER(Material), C.POINTER(C.POINTER(Wellbore))]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    """address of a numpy array or torch tensor (host or device)"""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    assert a.flags["C_CONTIGUOUS"]
    return C.c_void_p(a.ctypes.data)


def _np_ptr(a, t):
    return a.ctypes.data_as(t)


def color_elements(connects, n_nodes, nn=9):
    """host greedy colouring (SetUpColoredIndexes) of elements with nn connects;
    returns (n_colors, colours)"""
    connects = np.ascontiguousarray(connects, dtype=np.int32)
    col = np.zeros(connects.size // nn, np.int32)
    nc = lib().ipfem_color_elements_nn(col.size, int(n_nodes), int(nn), _np_ptr(connects, _ip), _np_ptr(col, _ip))
    if nc < 0:
        raise IpfemError(5, "bad colouring arguments")
    return int(nc), col


def wellbore_params(n, **kw):
    p = WellboreParams()
    lib().ipfem_wellbore_default(C.byref(p), int(n))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class _OwnedArray(np.ndarray):
    """an ndarray view of library memory that holds a reference to its owner"""

    def __array_finalize__(self, obj):
        self.owner = getattr(obj, "owner", None)


class WellboreMesh:
    """Quarter-annulus wellbore mesh provider (stand-in for the NeoPZ mesh)."""

    def __init__(self, params):
        self.params = params
        self._w = C.POINTER(Wellbore)()
        st = lib().ipfem_wellbore_build(C.byref(params), C.byref(self._w))
        if st != 0:
            raise IpfemError(st, "wellbore mesh build failed")
        w = self._w.contents
        self.n_el = w.mesh.n_elements
        self.n_nodes = w.mesh.n_nodes
        self.neq = 2 * self.n_nodes
        self.order = 2

    @property
    def mesh(self):
        return self._w.contents.mesh

    @property
    def material(self):
        return self._w.contents.material

    def array(self, name):
        """numpy view of one of the problem's arrays; the view (and every view
        derived from it) keeps the problem alive"""
        w = self._w.contents
        nn = (self.order + 1) ** 2
        n = {"node_xy": 2 * self.n_nodes, "connects": nn * self.n_el, "dphi": 2 * nn * nn * self.n_el,
             "weight": nn * self.n_el, "f0": self.neq, "df": self.neq, "fixed": self.neq,
             "el_cohesion": self.n_el, "el_phi": self.n_el, "el_shape": self.n_el}[name]
        p = getattr(w, name)
        if not p:
            return None
        a = np.ctypeslib.as_array(p, shape=(n,)).view(_OwnedArray)
        a.owner = self
        return a

    def close(self):
        if self._w:
            lib().ipfem_wellbore_free(self._w)
            self._w = C.POINTER(Wellbore)()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GmshMesh:
    """A Gmsh 4.1 mesh as the reference reads it (TPZGmshReader, main.cpp:447-464):
    vertices, 4-node quadrilaterals, boundary lines and points with their
    physical tags, and the $PhysicalNames table (name -> (dim, tag))."""

    def __init__(self, path):
        self._g = C.POINTER(GmshData)()
        st = lib().ipfem_gmsh_read(os.fsencode(path), C.byref(self._g))
        if st != 0:
            raise IpfemError(st, lib().ipfem_last_error(None).decode())
        g = self._g.contents

        def arr(p, n):
            return np.ctypeslib.as_array(p, shape=(n,)).copy() if n else np.zeros(0, np.int32)

        self.xy = arr(g.xy, 2 * g.n_nodes).reshape(-1, 2) if g.n_nodes else np.zeros((0, 2))
        self.quads = arr(g.quads, 4 * g.n_quads).reshape(-1, 4)
        self.quad_phys = arr(g.quad_phys, g.n_quads)
        self.tris = arr(g.tris, 3 * g.n_tris).reshape(-1, 3)
        self.tri_phys = arr(g.tri_phys, g.n_tris)
        self.lines = arr(g.lines, 2 * g.n_lines).reshape(-1, 2)
        self.line_phys = arr(g.line_phys, g.n_lines)
        self.points = arr(g.points, g.n_points)
        self.point_phys = arr(g.point_phys, g.n_points)
        self.physical = {g.phys_name[i].decode(): (int(g.phys_dim[i]), int(g.phys_tag[i])) for i in range(g.n_phys)}

    def tag(self, name_or_tag):
        return self.physical[name_or_tag][1] if isinstance(name_or_tag, str) else int(name_or_tag)

    def close(self):
        if self._g:
            lib().ipfem_gmsh_free(self._g)
            self._g = C.POINTER(GmshData)()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GmshProblem(WellboreMesh):
    """Elastoplastic problem of order 1, 2 or 3 on a Gmsh mesh
    (CmeshElastoplasticity, main.cpp:546-601).  bcs: (physical name or tag,
    type, value...) with the reference's TBCData types: 0 u = 0, 1 traction
    (tx, ty), 3 directional Dirichlet (fix the components with non-zero
    value), 6 normal stress (value * outward normal).  Loads are applied at
    load factor 1; angles in degrees; domain: physical name or tag of the
    quadrilaterals (None: all)."""

    def __init__(self, gmsh, bcs, E, nu, cohesion, phi_deg, psi_deg=None, domain=None, sigma0=(0.0, 0.0, 0.0, 0.0),
                 order=2):
        self.params = None
        arr = (BC * max(1, len(bcs)))()
        for i, b in enumerate(bcs):
            v = list(b[2:]) + [0.0, 0.0]
            arr[i] = BC(gmsh.tag(b[0]), int(b[1]), (C.c_double * 2)(float(v[0]), float(v[1])))
        m = Material()
        m.E, m.nu, m.cohesion = float(E), float(nu), float(cohesion)
        m.phi = np.deg2rad(float(phi_deg))
        m.psi = np.deg2rad(float(phi_deg if psi_deg is None else psi_deg))
        m.sigma0 = (C.c_double * 4)(*[float(x) for x in sigma0])
        self._w = C.POINTER(Wellbore)()
        dom = -1 if domain is None else gmsh.tag(domain)
        st = lib().ipfem_gmsh_problem(gmsh._g, int(order), int(dom), arr, len(bcs), C.byref(m), C.byref(self._w))
        if st != 0:
            raise IpfemError(st, lib().ipfem_last_error(None).decode())
        w = self._w.contents
        self.n_el = w.mesh.n_elements
        self.n_nodes = w.mesh.n_nodes
        self.neq = 2 * self.n_nodes
        self.order = int(w.mesh.order)
        self.n_ghost = int(w.n_ghost)
        self.n_equations = self.neq - 2 * self.n_ghost     # without the fixed ghost connects of triangles


class ElastoPlasticIntPointsStructMatrix:
    """Mirror of TPZElastoPlasticIntPointsStructMatrix over one ipfem context.

    Create()/CreateAssemble(rhs) build the integration-point data once;
    Assemble(K, rhs) computes tangent + residual, Assemble(rhs) the residual
    (TPZElastoPlasticIntPointsStructMatrix.cpp:34-78, 99-154).  The solution vector
    that the reference reads from the PZ mesh is passed explicitly.
    """

    def __init__(self, mesh, material=None, keep=None):
        if isinstance(mesh, WellboreMesh):
            keep, material, mesh = mesh, mesh.material, mesh.mesh
        self._keep = keep
        self._mesh = mesh
        self._material = material
        self._ctx = C.c_void_p()
        st = lib().ipfem_create(C.byref(mesh), C.byref(material), C.byref(self._ctx))
        if st != 0:
            raise IpfemError(st, lib().ipfem_last_error(None).decode() or "ipfem_create failed")
        sz = np.zeros(6, np.int64)
        lib().ipfem_sizes(self._ctx, _np_ptr(sz, _lp))
        self.n_el, self.n_ip, self.n_nodes, self.neq, self.n_colors, self.n_blocks = map(int, sz)
        self.order = int(mesh.order) or 2
        self.u = np.zeros(self.neq)   # the solution the reference reads from fMesh->Solution()

    def _check(self, st):
        if st != 0:
            raise IpfemError(st, lib().ipfem_last_error(self._ctx).decode())

    def close(self):
        if self._ctx:
            lib().ipfem_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- reference API --------------------------------------------------
    def Create(self):
        return self

    def CreateAssemble(self, rhs):
        self.Assemble(self, rhs)
        return self

    def Clone(self):
        return ElastoPlasticIntPointsStructMatrix(self._mesh, self._material, self._keep)

    def Assemble(self, *args):
        """Assemble(K, rhs) or Assemble(rhs); rhs is filled in place."""
        if len(args) == 2:
            _, rhs = args
            self._check(lib().ipfem_assemble(self._ctx, _ptr(self.u), _ptr(rhs), HOST))
        else:
            (rhs,) = args
            self._check(lib().ipfem_assemble_residual(self._ctx, _ptr(self.u), _ptr(rhs), HOST))
        return rhs

    def SetUpdateMem(self, flag):
        self._check(lib().ipfem_set_update_mem(self._ctx, int(bool(flag))))

    def set_newton_accel(self, mode):
        """0: plain Newton iteration; 1: modified-Thomas acceleration (main.cpp:194-217)"""
        self._check(lib().ipfem_set_newton_accel(self._ctx, int(mode)))

    def set_newton_tangent(self, mode):
        """0: Assemble(K, rhs) every iteration; 1: initial stiffness, the K of the
        first assembly kept (the reference's logged runs: main.cpp:218-222 with
        AssembleResidual in place of the Assemble of main.cpp:229-233)"""
        self._check(lib().ipfem_set_newton_tangent(self._ctx, int(mode)))

    def set_inner_tolerance(self, mode, gamma=0.9, alpha=2.0, eta_min=1e-5, eta_max=0.1):
        """0: every inner solve to cg_rtol; 1: adaptive forcing term (Eisenstat-Walker
        choice 2 with Kelley's safeguards), the first solve of a step to cg_rtol"""
        self._check(lib().ipfem_set_inner_tolerance(self._ctx, int(mode), float(gamma), float(alpha),
                                                     float(eta_min), float(eta_max)))

    def set_consistent_tangent(self, on):
        """1: the consistent spectral tangent (spin factors from the projected
        principal stresses); 0 (default): the reference's TangentOperator"""
        self._check(lib().ipfem_set_consistent_tangent(self._ctx, int(bool(on))))

    def set_spectral_mode(self, mode):
        """0 (default): the reference's spectral decomposition; 1: the closed
        form of plane-strain tensors, orthonormal at any eigenvalue gap"""
        self._check(lib().ipfem_set_spectral_mode(self._ctx, int(mode)))

    def set_newton_predictor(self, on):
        """1: each load step after the first starts from the secant prediction
        u + (u - u_prev); the convergence target stays |R| at the unpredicted start"""
        self._check(lib().ipfem_set_newton_predictor(self._ctx, int(bool(on))))

    def set_row_stencils(self, on):
        """1 (default): SpMVs form block columns from row stencils where the
        layout has them; 0: from the stored column indices (same result)"""
        self._check(lib().ipfem_set_row_stencils(self._ctx, int(bool(on))))

    def row_stencil_count(self):
        """(stencils of the FP64 layout, of the FP32 layout); 0 = explicit columns"""
        a, b = C.c_int32(0), C.c_int32(0)
        self._check(lib().ipfem_row_stencil_count(self._ctx, C.byref(a), C.byref(b)))
        return a.value, b.value

    def layout_info(self, fp32=False):
        """(stored 2x2 blocks, padded SELL slots, upper_only) of the tangent
        layout the SpMVs read now: the FP64 one, or with fp32 the FP32 one"""
        nb, ns, up = C.c_int64(0), C.c_int64(0), C.c_int32(0)
        self._check(lib().ipfem_layout_info(self._ctx, int(bool(fp32)), C.byref(nb), C.byref(ns), C.byref(up)))
        return nb.value, ns.value, bool(up.value)

    def set_precision(self, mode):
        self._check(lib().ipfem_set_precision(self._ctx, int(mode)))

    def set_residual_precision(self, bits, switch_rtol=1e-5):
        """32: FP32 strain gather / residual scatter in IPFEM_MIXED, with FP64
        refinement once |R| <= switch_rtol |R0| or |R| stops halving; 64: FP64"""
        self._check(lib().ipfem_set_residual_precision(self._ctx, int(bits), float(switch_rtol)))

    def SetLoadFactor(self, lam):
        self._check(lib().ipfem_set_load_factor(self._ctx, float(lam)))

    # -- extras -----------------------------------------------------------
    def assemble_residual(self, u, rhs, where=HOST):
        self._check(lib().ipfem_assemble_residual(self._ctx, _ptr(u), _ptr(rhs), where))
        return rhs

    def assemble(self, u, rhs, where=HOST):
        self._check(lib().ipfem_assemble(self._ctx, _ptr(u), _ptr(rhs), where))
        return rhs

    def stiffness(self):
        rp = np.zeros(self.n_nodes + 1, np.int64)
        col = np.zeros(self.n_blocks, np.int32)
        val = np.zeros(4 * self.n_blocks)
        self._check(lib().ipfem_get_stiffness(self._ctx, _np_ptr(rp, _lp), _np_ptr(col, _ip), _np_ptr(val, _dp)))
        return rp, col, val

    def stiffness_sym_csr(self):
        """K as TPZSYsmpMatrix stores it: upper-triangle CSR (IA, JA, A) over dofs"""
        nnz = np.zeros(1, np.int64)
        self._check(lib().ipfem_get_stiffness_sym_csr(self._ctx, _np_ptr(nnz, _lp), None, None, None))
        ia = np.zeros(self.neq + 1, np.int64)
        ja = np.zeros(int(nnz[0]), np.int64)
        a = np.zeros(int(nnz[0]))
        self._check(lib().ipfem_get_stiffness_sym_csr(self._ctx, _np_ptr(nnz, _lp), _np_ptr(ia, _lp),
                                                       _np_ptr(ja, _lp), _np_ptr(a, _dp)))
        return ia, ja, a

    def solve(self, b, x=None, rtol=1e-8, max_it=200000, where=HOST, allow_nonconverged=False):
        if x is None:
            x = np.zeros(self.neq)
        it = C.c_int()
        st = lib().ipfem_solve(self._ctx, _ptr(b), _ptr(x), float(rtol), int(max_it), where, C.byref(it))
        if not (allow_nonconverged and st == 1):
            self._check(st)
        return x, it.value

    def newton(self, u, n_steps, step_begin=0, step_end=None, newton_rtol=1e-8, newton_max_it=20, cg_rtol=1e-8,
               cg_max_it=200000, where=HOST, log_cap=4096, allow_nonconverged=True):
        if step_end is None:
            step_end = n_steps
        o = SolveOpts(int(n_steps), float(newton_rtol), int(newton_max_it), float(cg_rtol), int(cg_max_it))
        st = SolveStats()
        log = np.zeros(3 * log_cap)
        s = lib().ipfem_newton_solve(self._ctx, C.byref(o), int(step_begin), int(step_end), _ptr(u), where,
                                     C.byref(st), _np_ptr(log, _dp), int(log_cap))
        if not (allow_nonconverged and s == 1):
            self._check(s)
        return st, log[:3 * min(st.newton_iters, log_cap)].reshape(-1, 3)

    def newton_begin(self, n_steps, step_begin=0, step_end=None, newton_rtol=1e-8, newton_max_it=20, cg_rtol=1e-8,
                     cg_max_it=200000):
        if step_end is None:
            step_end = n_steps
        o = SolveOpts(int(n_steps), float(newton_rtol), int(newton_max_it), float(cg_rtol), int(cg_max_it))
        self._check(lib().ipfem_newton_begin(self._ctx, C.byref(o), int(step_begin), int(step_end)))

    def newton_advance(self, u, n_iters, where=HOST, log_cap=256):
        st = SolveStats()
        log = np.zeros(3 * log_cap)
        n = C.c_int32()
        self._check(lib().ipfem_newton_advance(self._ctx, int(n_iters), _ptr(u), where, C.byref(st),
                                               _np_ptr(log, _dp), int(log_cap), C.byref(n)))
        return st, log[:3 * min(n.value, log_cap)].reshape(-1, 3)

    def dot(self, d_a, d_b):
        out = np.zeros(1)
        self._check(lib().ipfem_dot(self._ctx, _ptr(d_a), _ptr(d_b), _np_ptr(out, _dp)))
        return float(out[0])

    def set_iteration_log(self, path):
        """append a JSON-lines record per Newton iteration and per accepted
        load step to `path` (None closes the log)"""
        self._check(lib().ipfem_set_iteration_log(self._ctx, os.fsencode(path) if path else None))

    @property
    def launch_count(self):
        return int(lib().ipfem_launch_count(self._ctx))

    def profile_spmv(self, reps=20):
        out = np.zeros(1)
        self._check(lib().ipfem_profile_spmv(self._ctx, int(reps), _np_ptr(out, _dp)))
        return float(out[0])

    def profile_residual(self, d_u, bits=64, reps=10):
        """CUDA-event durations (ms) of the residual kernels at the device
        displacement d_u: gather, return mapping, stress to element forces,
        colour reduction; bits 32 times the FP32 gather and scatter"""
        out = np.zeros(4)
        self._check(lib().ipfem_profile_residual(self._ctx, _ptr(d_u), int(bits), int(reps), _np_ptr(out, _dp)))
        return dict(zip(("gather_strain", "compute_sigma", "stress_residual", "color_reduce"), map(float, out)))

    # -- learned preconditioner --------------------------------------------
    def set_node_grid(self, gr, gt):
        self._check(lib().ipfem_set_node_grid(self._ctx, int(gr), int(gt)))

    def mlp_init(self, seed=0):
        self._check(lib().ipfem_mlp_init(self._ctx, int(seed)))

    def set_preconditioner(self, kind):
        self._check(lib().ipfem_set_preconditioner(self._ctx, int(kind)))

    def mlp_params(self):
        out = np.zeros(MLP_PARAMS, np.float32)
        self._check(lib().ipfem_mlp_get_params(self._ctx, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def set_mlp_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == MLP_PARAMS
        self._check(lib().ipfem_mlp_set_params(self._ctx, p.ctypes.data_as(C.POINTER(C.c_float))))

    def mlp_features(self, d_X):
        """features [n_nodes][32] of the current FP32 tangent into a device array"""
        self._check(lib().ipfem_mlp_features(self._ctx, _ptr(d_X)))

    def mlp_forward(self, d_X, rows, d_O):
        """network output [rows][20] of device feature rows [rows][32]"""
        self._check(lib().ipfem_mlp_forward(self._ctx, _ptr(d_X), int(rows), _ptr(d_O)))

    def mlp_operator(self, d_M):
        """the triangular factor G[5][n_nodes][2][2] of the current tangent (device)"""
        self._check(lib().ipfem_mlp_operator(self._ctx, _ptr(d_M)))

    def learn_grad(self, d_r, d_e, n_pairs, w_kaporin=1.0, w_pairs=1.0):
        """loss and parameter gradient: Kaporin term plus the (residual, increment)
        pairs [n_pairs][neq] (FP32, device; None with n_pairs = 0)"""
        g = np.zeros(MLP_PARAMS, np.float32)
        loss = np.zeros(1, np.float32)
        self._check(lib().ipfem_learn_grad(self._ctx, _ptr(d_r) if d_r is not None else None,
                                           _ptr(d_e) if d_e is not None else None, int(n_pairs),
                                           float(w_kaporin), float(w_pairs),
                                           g.ctypes.data_as(C.POINTER(C.c_float)),
                                           loss.ctypes.data_as(C.POINTER(C.c_float))))
        return g, float(loss[0])

    def mlp_adam(self, grads, lr):
        """one Adam step with a host gradient (None: the context's last gradient)"""
        if grads is None:
            self._check(lib().ipfem_mlp_adam(self._ctx, None, float(lr)))
        else:
            g = np.ascontiguousarray(grads, dtype=np.float32)
            assert g.size == MLP_PARAMS
            self._check(lib().ipfem_mlp_adam(self._ctx, g.ctypes.data_as(C.POINTER(C.c_float)), float(lr)))

    def cg_snapshots(self, d_b, snap_iters, d_xs, d_rs, d_xfinal, rtol=1e-6, max_it=200000):
        si = np.ascontiguousarray(snap_iters, dtype=np.int32)
        it = C.c_int()
        self._check(lib().ipfem_cg_snapshots(self._ctx, _ptr(d_b), float(rtol), int(max_it), int(si.size),
                                             si.ctypes.data_as(_ip), _ptr(d_xs), _ptr(d_rs), _ptr(d_xfinal),
                                             C.byref(it)))
        return it.value

    def measure_fp64_peak(self):
        out = np.zeros(1)
        self._check(lib().ipfem_measure_fp64_peak(self._ctx, _np_ptr(out, _dp)))
        return float(out[0])

    def gather_strain(self, d_u, d_strain):
        self._check(lib().ipfem_gather_strain(self._ctx, _ptr(d_u), _ptr(d_strain)))

    def compute_sigma(self, update_mem, d_strain, d_sigma_w, d_dep=None):
        self._check(lib().ipfem_compute_sigma(self._ctx, int(update_mem), _ptr(d_strain), _ptr(d_sigma_w),
                                              _ptr(d_dep)))

    def scatter_residual(self, d_sigma_w, d_res):
        self._check(lib().ipfem_scatter_residual(self._ctx, _ptr(d_sigma_w), _ptr(d_res)))

    def gather_strain32(self, d_u, d_strain32):
        """FP32 strain gather (MIXED with FP32 residuals): float32 [3][n_ip]"""
        self._check(lib().ipfem_gather_strain32(self._ctx, _ptr(d_u), _ptr(d_strain32)))

    def scatter_residual32(self, d_sigma_w32, d_res):
        """FP32 element forces and colour sums from float32 [3][n_ip] into FP64 d_res"""
        self._check(lib().ipfem_scatter_residual32(self._ctx, _ptr(d_sigma_w32), _ptr(d_res)))

    def get_state(self, field):
        n = {0: 4 * self.n_ip, 1: 4 * self.n_ip, 2: self.n_ip, 3: self.n_ip}[field]
        out = np.zeros(n)
        self._check(lib().ipfem_get_state(self._ctx, int(field), _np_ptr(out, _dp)))
        return out

    def set_state(self, field, arr):
        arr = np.ascontiguousarray(arr, dtype=np.float64)
        self._check(lib().ipfem_set_state(self._ctx, int(field), _np_ptr(arr, _dp)))

    def save_checkpoint(self, path, u, step):
        """write u (host or device) and the committed integration-point state
        (plastic strain, stress, alpha, m_type) after load step `step` to an
        .npz file; load_checkpoint restores them into a context of the same
        problem, from which the load-stepped solve continues with the same
        iterates (the reference keeps this state only in memory,
        TPZConstitutiveLawProcessor.cpp:86-121)"""
        uh = u.detach().cpu().numpy() if hasattr(u, "detach") else np.asarray(u)
        np.savez(path, u=np.asarray(uh, dtype=np.float64), step=np.int64(step), neq=np.int64(self.neq),
                 **{"state%d" % f: self.get_state(f) for f in range(4)})

    def load_checkpoint(self, path):
        """restore a save_checkpoint file; returns (u as a host array, step)"""
        d = np.load(path)
        if int(d["neq"]) != self.neq:
            raise IpfemError(5, "checkpoint of a problem with %d equations, this one has %d" % (int(d["neq"]),
                                                                                               self.neq))
        for f in range(4):
            self.set_state(f, d["state%d" % f])
        return np.array(d["u"]), int(d["step"])

    def get_setup(self, field):
        nn = self.n_ip // self.n_el
        spec = {0: (self.n_el, np.int32), 1: (1, np.int32), 2: (2 * nn * self.n_el, np.int32),
                3: (2 * nn * nn * self.n_el, np.float64), 4: (self.n_ip, np.float64)}[field]
        out = np.zeros(spec[0], spec[1])
        self._check(lib().ipfem_get_setup(self._ctx, int(field), C.c_void_p(out.ctypes.data)))
        return out

    @property
    def stream(self):
        return lib().ipfem_stream(self._ctx)
