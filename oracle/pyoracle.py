"""ctypes view of the CPU oracle (test infrastructure only).

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg,
never by the product package.
"""
import contextlib
import ctypes as C
import os

import numpy as np

from . import build as _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_lp = C.POINTER(C.c_int64)
_bp = C.POINTER(C.c_uint8)


class Params(C.Structure):
    _fields_ = [("nr", C.c_int32), ("nt", C.c_int32), ("r_in", C.c_double), ("r_out", C.c_double),
                ("grading", C.c_double), ("E", C.c_double), ("nu", C.c_double),
                ("cohesion", C.c_double), ("phi_deg", C.c_double), ("psi_deg", C.c_double),
                ("sxx0", C.c_double), ("syy0", C.c_double), ("sxy0", C.c_double), ("szz0", C.c_double),
                ("pw_final", C.c_double), ("material_mode", C.c_int32), ("c_cv", C.c_double),
                ("phi_lo_deg", C.c_double), ("phi_hi_deg", C.c_double), ("seed", C.c_uint64)]


class MC(C.Structure):
    _fields_ = [("cohesion", C.c_double), ("sinphi", C.c_double), ("cosphi", C.c_double),
                ("tanphi", C.c_double), ("sinpsi", C.c_double)]


class Elastic(C.Structure):
    _fields_ = [("lam", C.c_double), ("mu", C.c_double)]


class Problem(C.Structure):
    _fields_ = [("prm", Params), ("n_el", C.c_int32), ("n_nodes", C.c_int32), ("neq", C.c_int32),
                ("n_ip", C.c_int64), ("node_xy", _dp), ("connects", _ip), ("fixed", _bp),
                ("f0", _dp), ("df", _dp), ("el", Elastic), ("mats", C.POINTER(MC)), ("eps_p0", _dp),
                ("B", _dp), ("weight", _dp), ("dofs", _ip), ("n_colors", C.c_int32),
                ("el_color", _ip), ("color_ptr", _ip), ("color_els", _ip), ("n_blocks", C.c_int64),
                ("row_ptr", _lp), ("col", _ip), ("el_blk", _lp), ("eps_p", _dp), ("sigma", _dp),
                ("mtype", C.POINTER(C.c_int8)), ("alpha", _dp), ("strain", _dp), ("sigma_w", _dp),
                ("dep", _dp), ("K", _dp), ("dinv", _dp), ("nthreads", C.c_int), ("order", C.c_int32),
                ("nn", C.c_int32), ("nq", C.c_int32), ("nd", C.c_int32), ("binv", _dp), ("cg_block", C.c_int32),
                ("ext_dphi", _dp), ("ext_weight", _dp)]


class SolveOpts(C.Structure):
    _fields_ = [("n_steps", C.c_int32), ("newton_rtol", C.c_double), ("newton_max_it", C.c_int32),
                ("cg_rtol", C.c_double), ("cg_max_it", C.c_int32), ("accel", C.c_int32),
                ("tangent_mode", C.c_int32)]


class MeshIn(C.Structure):
    _fields_ = [("n_el", C.c_int32), ("n_nodes", C.c_int32), ("node_xy", _dp), ("connects", _ip),
                ("fixed", _bp), ("f0", _dp), ("df", _dp), ("order", C.c_int32), ("dphi", _dp), ("weight", _dp)]


class SolveStats(C.Structure):
    _fields_ = [("newton_iters", C.c_int32), ("cg_iters", C.c_int64), ("last_step_iters", C.c_int32),
                ("converged", C.c_int32), ("final_res", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        so = _build.build_oracle()
        L = C.CDLL(so)
        L.orc_problem_create.restype = C.POINTER(Problem)
        L.orc_problem_create.argtypes = [C.POINTER(Params), C.c_int]
        L.orc_problem_from_mesh.restype = C.POINTER(Problem)
        L.orc_problem_from_mesh.argtypes = [C.POINTER(MeshIn), C.POINTER(Params), C.c_int]
        L.orc_problem_destroy.argtypes = [C.POINTER(Problem)]
        L.orc_default_params.argtypes = [C.POINTER(Params), C.c_int]
        L.orc_dot.restype = C.c_double
        L.orc_dot.argtypes = [C.c_int64, _dp, _dp]
        L.orc_dot_final.restype = C.c_double
        L.orc_dot_final.argtypes = [C.c_int64, _dp]
        L.orc_dot_partials.restype = C.c_int64
        L.orc_dot_partials.argtypes = [C.c_int64, _dp, _dp, _dp]
        L.orc_assemble_residual.argtypes = [C.POINTER(Problem), _dp, C.c_double, C.c_int, _dp]
        L.orc_assemble.argtypes = [C.POINTER(Problem), _dp, C.c_double, _dp]
        L.orc_spmv.argtypes = [C.POINTER(Problem), _dp, _dp]
        L.orc_pcg.restype = C.c_int
        L.orc_pcg.argtypes = [C.POINTER(Problem), _dp, _dp, C.c_double, C.c_int, _dp]
        L.orc_gather_strain.argtypes = [C.POINTER(Problem), _dp, _dp]
        L.orc_scatter_residual.argtypes = [C.POINTER(Problem), _dp, _dp]
        L.orc_solve_steps.argtypes = [C.POINTER(Problem), C.POINTER(SolveOpts), C.c_int32, C.c_int32,
                                      _dp, C.POINTER(SolveStats), _dp, C.c_int32]
        L.orc_mc_from_angles.argtypes = [C.c_double, C.c_double, C.c_double, C.POINTER(MC)]
        L.orc_lame_from_engineering.argtypes = [C.c_double, C.c_double, C.POINTER(Elastic)]
        L.orc_ip_update.argtypes = [C.POINTER(Elastic), C.POINTER(MC), _dp, _dp, C.c_double, _dp, _dp,
                                    _dp, _dp, _dp, C.POINTER(C.c_int), _dp]
        L.orc_ip_update_gpu_alias.argtypes = [C.POINTER(Elastic), C.POINTER(MC), _dp, _dp, C.c_double,
                                              _dp, _dp, _dp, C.POINTER(C.c_int), _dp]
        L.orc_compute_sigma_batch.argtypes = [C.c_int64, C.c_int, C.POINTER(Elastic), C.POINTER(MC), _dp,
                                              _dp, _dp, C.c_int, _dp, _dp, _dp, C.POINTER(C.c_int8), _dp]
        L.orc_set_consistent_tangent.argtypes = [C.c_int]
        L.orc_spectral.argtypes = [_dp, _dp, _dp]
        L.orc_set_spectral_mode.argtypes = [C.c_int]
        L.orc_greedy_coloring.restype = C.c_int32
        L.orc_greedy_coloring.argtypes = [C.c_int32, C.c_int32, _ip, _ip]
        _lib = L
    return _lib


def ptr(a):
    """data pointer of a contiguous numpy array, typed for ctypes"""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    t = {np.float64: _dp, np.int32: _ip, np.int64: _lp, np.uint8: _bp, np.int8: C.POINTER(C.c_int8)}[a.dtype.type]
    return a.ctypes.data_as(t)


def default_params(n, **kw):
    p = Params()
    lib().orc_default_params(C.byref(p), int(n))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _view(p, n, dtype):
    return np.ctypeslib.as_array(p, shape=(int(n),)).view(dtype) if n else np.zeros(0, dtype)


class OracleProblem:
    """Owns an orc_problem; numpy views of its arrays (valid while alive)."""

    def __init__(self, params, nthreads=0, mesh=None):
        """the structured quarter annulus of `params`, or with mesh = dict(node_xy,
        connects, fixed, f0, df[, order][, dphi, weight]) a caller's mesh of order
        1, 2 or 3, its element blocks computed from the coordinates or given
        (params then give the material and in-situ stress only)"""
        self.params = params
        if mesh is None:
            self._p = lib().orc_problem_create(C.byref(params), int(nthreads))
        else:
            a = {k: np.ascontiguousarray(mesh[k], dtype=t) for k, t in
                 (("node_xy", np.float64), ("connects", np.int32), ("fixed", np.uint8), ("f0", np.float64),
                  ("df", np.float64))}
            order = int(mesh.get("order", 2))
            ext = {k: np.ascontiguousarray(mesh[k], dtype=np.float64) for k in ("dphi", "weight") if k in mesh}
            m = MeshIn(a["connects"].size // (order + 1) ** 2, a["node_xy"].size // 2, ptr(a["node_xy"]),
                       ptr(a["connects"]), ptr(a["fixed"]), ptr(a["f0"]), ptr(a["df"]), order,
                       ptr(ext.get("dphi")), ptr(ext.get("weight")))
            self._p = lib().orc_problem_from_mesh(C.byref(m), C.byref(params), int(nthreads))
        P = self._p.contents
        self.P = P
        self.n_el, self.n_nodes, self.neq, self.n_ip = P.n_el, P.n_nodes, P.neq, P.n_ip
        self.order, self.nn, self.nq, self.nd = P.order, P.nn, P.nq, P.nd
        self.n_colors = P.n_colors
        self.n_blocks = P.n_blocks

    def close(self):
        if self._p:
            lib().orc_problem_destroy(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # array views
    def arr(self, name):
        P = self.P
        nn, nq, nd = self.nn, self.nq, self.nd
        sizes = {"node_xy": (2 * self.n_nodes, np.float64), "connects": (nn * self.n_el, np.int32),
                 "fixed": (self.neq, np.uint8), "f0": (self.neq, np.float64), "df": (self.neq, np.float64),
                 "B": (3 * nq * nd * self.n_el, np.float64), "weight": (self.n_ip, np.float64),
                 "dofs": (nd * self.n_el, np.int32), "el_color": (self.n_el, np.int32),
                 "color_ptr": (self.n_colors + 1, np.int32), "color_els": (self.n_el, np.int32),
                 "row_ptr": (self.n_nodes + 1, np.int64), "col": (self.n_blocks, np.int32),
                 "el_blk": (nn * nn * self.n_el, np.int64), "eps_p": (6 * self.n_ip, np.float64),
                 "sigma": (6 * self.n_ip, np.float64), "mtype": (self.n_ip, np.int8),
                 "alpha": (self.n_ip, np.float64), "strain": (3 * self.n_ip, np.float64),
                 "sigma_w": (3 * self.n_ip, np.float64), "dep": (9 * self.n_ip, np.float64),
                 "K": (4 * self.n_blocks, np.float64), "dinv": (self.neq, np.float64),
                 "eps_p0": (6, np.float64), "binv": (4 * self.n_nodes, np.float64)}
        n, dt = sizes[name]
        return np.ctypeslib.as_array(getattr(P, name), shape=(int(n),))

    def mats(self):
        P = self.P
        m = np.ctypeslib.as_array(C.cast(P.mats, _dp), shape=(5 * self.n_el,)).reshape(self.n_el, 5)
        return m  # columns: cohesion, sinphi, cosphi, tanphi, sinpsi

    def assemble_residual(self, u, lam, update_mem=False):
        rhs = np.zeros(self.neq)
        lib().orc_assemble_residual(self._p, ptr(u), float(lam), int(update_mem), ptr(rhs))
        return rhs

    def assemble(self, u, lam):
        rhs = np.zeros(self.neq)
        lib().orc_assemble(self._p, ptr(u), float(lam), ptr(rhs))
        return rhs

    def spmv(self, x):
        y = np.zeros(self.neq)
        lib().orc_spmv(self._p, ptr(x), ptr(y))
        return y

    def set_block_jacobi(self, on=True):
        """precondition orc_pcg (and the Newton solve) with the nodal block-Jacobi inverse"""
        self.P.cg_block = 1 if on else 0

    def pcg(self, b, rtol=1e-8, max_it=100000):
        x = np.zeros(self.neq)
        work = np.zeros(4 * self.neq)
        k = lib().orc_pcg(self._p, ptr(np.ascontiguousarray(b)), ptr(x), float(rtol), int(max_it), ptr(work))
        return x, k

    def solve_steps(self, u, n_steps, step_begin=0, step_end=None, newton_rtol=1e-8, newton_max_it=20,
                    cg_rtol=1e-8, cg_max_it=200000, log_cap=4096, accel=0, tangent_mode=0):
        if step_end is None:
            step_end = n_steps
        o = SolveOpts(int(n_steps), float(newton_rtol), int(newton_max_it), float(cg_rtol), int(cg_max_it),
                      int(accel), int(tangent_mode))
        st = SolveStats()
        log = np.zeros(3 * log_cap)
        lib().orc_solve_steps(self._p, C.byref(o), int(step_begin), int(step_end), ptr(u), C.byref(st),
                              ptr(log), int(log_cap))
        nlog = st.newton_iters
        return st, log[:3 * min(nlog, log_cap)].reshape(-1, 3)


@contextlib.contextmanager
def plane_spectral():
    """The oracle's closed-form plane-strain spectral decomposition
    (orc_set_spectral_mode(1)) for the duration of the block; the reference's
    decomposition is restored on exit."""
    lib().orc_set_spectral_mode(1)
    try:
        yield
    finally:
        lib().orc_set_spectral_mode(0)


@contextlib.contextmanager
def consistent_tangent():
    """The oracle's consistent spectral tangent (orc_set_consistent_tangent)
    for the duration of the block.  The switch is global to the process; the
    reference's tangent is restored on exit."""
    lib().orc_set_consistent_tangent(1)
    try:
        yield
    finally:
        lib().orc_set_consistent_tangent(0)


def dot(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return lib().orc_dot(a.size // 2, ptr(a), ptr(b))


class OracleNewton:
    """Resumable form of orc_solve_steps (plain Newton, full tangent), cut into
    Newton iterations exactly as the library's ipfem_newton_advance cuts them:
    an iteration is CG on the current tangent, u += du, Assemble(K, rhs) and
    the convergence test; a load step that converges (or reaches
    newton_max_it) is accepted inside the iteration that ends it (state
    commit, main.cpp:487-522), and the next step's first assembly opens the
    following iteration (main.cpp:160-262).  Same calls in the same order as
    orc_solve_steps, so the iterates are identical."""

    def __init__(self, prob, n_steps, step_begin=0, step_end=None, newton_rtol=1e-8, newton_max_it=20,
                 cg_rtol=1e-8, cg_max_it=200000):
        self.p = prob
        self.n_steps = int(n_steps)
        self.step = int(step_begin)
        self.step_end = self.n_steps if step_end is None else int(step_end)
        self.newton_rtol, self.newton_max_it = float(newton_rtol), int(newton_max_it)
        self.cg_rtol, self.cg_max_it = float(cg_rtol), int(cg_max_it)
        self.open = False
        self.R = None
        self.r0 = self.rn = 0.0
        self.it = 0
        self.all_converged = True

    def _lam(self):
        return (self.step + 1) / self.n_steps

    def advance(self, u, n_iters=0):
        """n_iters Newton iterations on u (in place; 0 = to the end of the last
        step); returns (iterations, CG iterations) performed"""
        done, cg = 0, 0
        n_iters = n_iters or (1 << 30)
        while done < n_iters and self.step < self.step_end:
            lam = self._lam()
            if not self.open:
                self.R = self.p.assemble(u, lam)
                self.r0 = self.rn = float(np.sqrt(dot(self.R, self.R)))
                self.it = 0
                self.open = True
            conv = self.r0 == 0.0
            if not conv:
                du, k = self.p.pcg(self.R, rtol=self.cg_rtol, max_it=self.cg_max_it)
                cg += abs(k)
                u += du
                self.it += 1
                done += 1
                self.R = self.p.assemble(u, lam)
                self.rn = float(np.sqrt(dot(self.R, self.R)))
                conv = self.rn <= self.newton_rtol * self.r0
            if conv or self.it >= self.newton_max_it:
                if not conv:
                    self.all_converged = False
                self.p.assemble_residual(u, lam, update_mem=True)
                self.step += 1
                self.open = False
        return done, cg
