"""Benchmark: ms per Newton iteration (and residual IP/s) of the plain FP64
wellbore solve, 400 x 400 order-2 quads (1.44 M integration points,
1 283 202 dofs), block-Jacobi CG to 1e-8 and Newton to 1e-8 relative
residual, on one GB300 (--jacobi: scalar Jacobi).

A step is one Newton iteration of the load-stepped solve (CG on the current
tangent, u += du, Assemble(K, rhs), convergence test; load-step acceptance
and the next step's first assembly fall inside the iteration where they
occur).  W warm-up iterations run untimed, then exactly K are timed.

  value    : device-timed (CUDA events on the library's stream), inputs resident
  e2e      : the same iterations through the C-ABI with a pinned host u: each
             timed step is one ipfem_newton_advance(u, 1, IPFEM_HOST) call,
             which copies u H2D on entry and D2H on exit; host-timed
  solve    : time to solution: the whole load-stepped solve (the warm-up,
             timed and remaining iterations of the same run), with its Newton
             and CG iteration counts, for the plain and the chosen method
  roofline : the CG block SpMV (dominant kernel), algorithmic bytes / launch
             over its CUDA-event duration, against the measured HBM copy peak
  cpu_baseline : the C oracle on the host cores, bounded sample (one tangent
             assembly + S CG iterations with the same preconditioner), scaled to
             a Newton iteration with the CG iteration count this run measured on
             the GPU (the oracle performs bit-identical arithmetic, so the
             counts are the same)

--impl reference runs the oracle's own Newton iterations on all host cores:
the same W warm-up and K timed iterations of the same solve, measured, not
scaled (the reference's own CPU path cannot be built: it needs NeoPZ, Intel
MKL and TBB).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms/Newton iter & IP/s at 1e-8 rel residual, chosen vs plain FP64, 1 GB300"
UNIT = "ms/Newton iter"
N_STEPS = 20
# the configurations the metric is quoted on: mesh n x n, load steps, material
CONFIGS = {
    1: {"n": 40, "n_steps": 10, "wb": {}},
    2: {"n": 400, "n_steps": 20, "wb": {}},
    3: {"n": 1000, "n_steps": 20, "wb": {"material_mode": 1, "c_cv": 0.2}},
    4: {"n": 400, "n_steps": 20, "wb": {}},
    5: {"n": 2000, "n_steps": 30, "wb": {"material_mode": 2, "c_cv": 0.3, "phi_lo_deg": 25.0, "phi_hi_deg": 35.0,
                                         "pw_final": -5.0}},
}
# DRAM bytes (read + write) of one FP64 SpMV launch at 400 x 400 (rows sorted
# by length), from the ncu capture of that launch (dram__bytes_read.sum +
# dram__bytes_write.sum): with row stencils, and with the stored column indices
SPMV_DRAM_BYTES = {True: 346.375424e6 + 4.631552e6, False: 388.405504e6 + 9.274112e6}
FALLBACK_HBM_GBS = 6800.0


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def residual_kernel_roofline(M, ms, fp, hbm_peak):
    """algorithmic bytes of the residual kernels of struct matrix M (fp = 8:
    the FP64 kernels, 4: the FP32 gather and scatter) over their CUDA-event
    durations ms, against the measured HBM copy bandwidth.  Gather: element
    blocks, dof map, u once, strains; stress: blocks, weighted stresses,
    element forces; reduce: incidence, element forces, load vector, fixed, rhs.
    The return mapping is bound by the FP64 pipe and reported as a time."""
    nn = (M.order + 1) ** 2
    nb, nd = nn * 2 * nn, 2 * nn
    e, q, neq = M.n_el, M.n_ip, M.neq
    by = {"gather_strain": e * nb * fp + e * nd * 4 + neq * 8 + 3 * q * fp,
          "stress_residual": e * nb * fp + 3 * q * fp + e * nd * fp,
          "color_reduce": M.n_colors * M.n_nodes * 4 + e * nd * fp + neq * (8 + 1 + 8)}
    out = {}
    for k, b in by.items():
        gbs = b / (ms[k] * 1e-3) / 1e9
        out[k] = {"ms": ms[k], "algorithmic_bytes": b, "achieved_gbs": gbs, "frac": gbs / hbm_peak}
    out["compute_sigma"] = {"ms": ms["compute_sigma"], "bound": "fp64 pipe"}
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms"""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


class CpuArm:
    """The C oracle on the host cores (bounded samples of the same workload)."""

    def __init__(self, n, threads, n_steps=N_STEPS, wb=None, block=True):
        import numpy as np

        from oracle import pyoracle as po

        self.n = n
        self.threads = threads
        t0 = time.perf_counter()
        self.P = po.OracleProblem(po.default_params(n, **(wb or {})), nthreads=threads)
        self.P.set_block_jacobi(block)
        self.n_steps = n_steps
        self.t_setup = time.perf_counter() - t0
        self.u = np.zeros(self.P.neq)

    def sample(self, cg_per_iter, cg_sample):
        """one tangent assembly + cg_sample CG iterations + one residual,
        scaled to a Newton iteration of cg_per_iter CG iterations"""
        lam = 1.0 / self.n_steps
        t0 = time.perf_counter()
        R = self.P.assemble(self.u, lam)
        t_asm = time.perf_counter() - t0
        t0 = time.perf_counter()
        self.P.assemble_residual(self.u, lam)
        t_res = time.perf_counter() - t0
        t0 = time.perf_counter()
        _, k = self.P.pcg(R, rtol=1e-8, max_it=cg_sample)
        t_cg = (time.perf_counter() - t0) / max(1, abs(k))
        return {"ms_per_newton": 1e3 * (t_asm + t_cg * cg_per_iter), "t_asm_ms": 1e3 * t_asm,
                "t_cg_iter_ms": 1e3 * t_cg, "t_res_ms": 1e3 * t_res, "ip_per_s": self.P.n_ip / t_res,
                "cg_sample": abs(k)}

    def close(self):
        self.P.close()


def reduce_max(x, dist=None):
    """max of a per-rank float over all ranks (identity without a process group)"""
    if dist is None or not dist.is_initialized():
        return x
    import torch

    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def ddp_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload_config(args):
    """the workload both arms run, named by what it is (identical dicts)"""
    n = args.n
    n_ip, neq = 9 * n * n, 2 * (2 * n + 1) ** 2
    n_blocks = (8 * n + 1) ** 2
    prec = "Jacobi-CG" if args.jacobi else "block-Jacobi CG"
    return {"workload": "wellbore %dx%d order-2 quads, %d IPs, %d dofs, plain FP64, %s 1e-8, Newton 1e-8, "
                        "%d load steps%s; Newton iterations %d-%d of the solve timed (warm-up %d)"
                        % (n, n, n_ip, neq, prec, args.n_steps,
                           (", material %s" % json.dumps(args.wb)) if args.wb else "",
                           args.warmup + 1, args.warmup + args.steps, args.warmup),
            "mesh": "%dx%d" % (n, n), "load_steps": args.n_steps, "ips": n_ip, "dofs": neq,
            "linear_solver": prec, "cg_rtol": 1e-8, "newton_rtol": 1e-8,
            "l2": ("inputs larger than L2 (tangent %.0f MB, element blocks %.0f MB)" if n_blocks * 32 > 129e6
                   else "inputs fit in L2 (tangent %.0f MB, element blocks %.0f MB); no flush")
                  % (n_blocks * 32 / 1e6, n * n * 1296 / 1e6)}


def run_reference(args):
    """The oracle's Newton iterations on all host cores: W untimed, K timed.
    The oracle's arithmetic is the library's bit for bit, so these are the
    same iterations (same CG counts) as the GPU arm's."""
    ws, rank, _ = ddp_env()
    if rank != 0:
        return 0
    import numpy as np

    from oracle import pyoracle as po

    threads = args.cpu_threads or os.cpu_count()
    P = po.OracleProblem(po.default_params(args.n, **args.wb), nthreads=threads)
    P.set_block_jacobi(not args.jacobi)
    u = np.zeros(P.neq)
    newton = po.OracleNewton(P, args.n_steps, newton_max_it=40, cg_rtol=1e-8)
    _, cg_w = newton.advance(u, args.warmup)
    t0 = time.perf_counter()
    k, cg = newton.advance(u, args.steps)
    t_run = time.perf_counter() - t0
    ms = 1e3 * t_run / max(1, k)
    # residual evaluation (Assemble(rhs)) at the reached state, for IP/s
    t0 = time.perf_counter()
    nres = 3
    for _ in range(nres):
        P.assemble_residual(u, newton._lam())
    t_res = (time.perf_counter() - t0) / nres
    P.close()
    line = {
        "impl": "reference", "metric": METRIC, "value": ms, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args),
        "ip_per_s": P.n_ip / t_res,
        "newton_iters_timed": k,
        "cg_iters_per_newton": cg / max(1, k),
        "cpu_baseline": {"value": ms, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "the C oracle's own Newton iterations %d-%d of the solve (tangent assembly, "
                                   "%s to 1e-8: %d CG iterations, residual norm and load-step commit), "
                                   "measured on %d host threads; residual evaluation %.1f ms"
                                   % (args.warmup + 1, args.warmup + k,
                                      "Jacobi-CG" if args.jacobi else "block-Jacobi CG", cg, threads,
                                      1e3 * t_res)},
        "e2e": {"value": ms, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def timed_advance(S, stream, u, n_iters, e0, e1):
    """n_iters Newton iterations (0 = to the end of the solve) of context S,
    CUDA-event timed on its stream; returns (stats, ms)"""
    import torch

    import intpointsfem_gb300 as ip

    torch.cuda.synchronize()
    e0.record(stream)
    st, _ = S.newton_advance(u, n_iters, ip.DEVICE)
    e1.record(stream)
    torch.cuda.synchronize()
    return st, e0.elapsed_time(e1)


def solve_record(parts, n_steps):
    """time to solution from the (stats, ms) of consecutive advances that
    together cover the whole load-stepped solve"""
    ms = sum(p[1] for p in parts)
    nit = sum(p[0].newton_iters for p in parts)
    cg = sum(p[0].cg_iters for p in parts)
    return {"ms": ms, "load_steps": n_steps, "newton_iters": nit, "cg_iters": cg,
            "ms_per_newton_iter": ms / max(1, nit), "converged": bool(parts[-1][0].converged),
            "fcg_fallbacks": sum(p[0].fcg_fallbacks for p in parts)}


def run_gpu(args):
    import numpy as np
    import torch

    ws, rank, local = ddp_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import __graft_entry__ as ge
    if rank == 0 or ws == 1:
        ge.build()
    if dist:
        dist.barrier()
    import intpointsfem_gb300 as ip

    dev = torch.device("cuda", local if ws > 1 else 0)
    torch.cuda.set_device(dev)
    n = args.n
    wb = ip.WellboreMesh(ip.wellbore_params(n, **args.wb))
    N_STEPS = args.n_steps
    mixed = args.precision == "mixed"
    if args.mixed_cg_rtol is None:
        args.mixed_cg_rtol = ip.CHOSEN_CG_RTOL if args.inner == "adaptive" else ip.FIXED_CG_RTOL
    cg_rtol = args.mixed_cg_rtol if mixed else 1e-8

    def set_inner(M):
        # the mixed methods' Newton settings: inner tolerance (adaptive forcing
        # term or fixed), the secant predictor of the load steps and the tangent
        if args.inner == "adaptive":
            M.set_inner_tolerance(**ip.CHOSEN_INNER)
        M.set_newton_predictor(args.predictor == "on")
        M.set_consistent_tangent(args.tangent == "consistent")
        M.set_spectral_mode(1 if args.spectral == "plane" else 0)

    A = ip.ElastoPlasticIntPointsStructMatrix(wb)         # device-resident arm
    if mixed:
        A.set_precision(ip.MIXED)
        set_inner(A)
        if args.residual32:
            A.set_residual_precision(32)
    if not args.jacobi:
        A.set_preconditioner(ip.PREC_BLOCK_JACOBI)
    if args.no_row_stencils:
        A.set_row_stencils(0)
    stream = torch.cuda.ExternalStream(A.stream, device=dev)
    fp64_tflops = A.measure_fp64_peak()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    # residual evaluation throughput (Assemble(rhs)), inputs resident
    du = torch.zeros(A.neq, dtype=torch.float64, device=dev)
    dr = torch.zeros_like(du)
    A.SetLoadFactor(1.0 / N_STEPS)
    for _ in range(3):
        A.assemble_residual(du, dr, ip.DEVICE)
    nres = 20
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(nres):
        A.assemble_residual(du, dr, ip.DEVICE)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_res = e0.elapsed_time(e1) / nres

    # Newton iterations, device-resident: W warm-up, K timed, then (for the
    # time to solution) the rest of the same solve
    A.newton_begin(N_STEPS, newton_max_it=40, cg_rtol=cg_rtol)
    part_w = timed_advance(A, stream, du, args.warmup, e0, e1)
    clocks = ClockSampler(dev.index)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    l0 = A.launch_count
    e0.record(stream)
    st, log = A.newton_advance(du, args.steps, ip.DEVICE)
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms_timed = e0.elapsed_time(e1)
    launches = A.launch_count - l0
    # per Newton iteration actually run (a short solve can end inside the window)
    n_timed = max(1, st.newton_iters)
    ms_dev = reduce_max(ms_timed / n_timed, dist)
    cg_per_iter = st.cg_iters / max(1, st.newton_iters)
    solve_plain = None
    if args.solve:
        part_r = timed_advance(A, stream, du, 0, e0, e1)
        solve_plain = solve_record([part_w, (st, ms_timed), part_r], N_STEPS)

    # e2e through the C-ABI with a pinned host u: one call per Newton
    # iteration, u copied H2D on entry and D2H on exit of every call
    ms_e2e = None
    if not args.no_e2e:
        B = ip.ElastoPlasticIntPointsStructMatrix(wb)
        if mixed:
            B.set_precision(ip.MIXED)
            set_inner(B)
        if not args.jacobi:
            B.set_preconditioner(ip.PREC_BLOCK_JACOBI)
        if args.no_row_stencils:
            B.set_row_stencils(0)
        hu = torch.zeros(B.neq, dtype=torch.float64, pin_memory=True)
        B.newton_begin(N_STEPS, newton_max_it=40, cg_rtol=cg_rtol)
        for _ in range(args.warmup):
            B.newton_advance(hu, 1, ip.HOST)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        n_e2e = 0
        for _ in range(args.steps):
            n_e2e += B.newton_advance(hu, 1, ip.HOST)[0].newton_iters
        ms_e2e = 1e3 * (time.perf_counter() - t0) / max(1, n_e2e)
        B.close()

    # the chosen method (mixed precision + learned preconditioner) and mixed
    # precision with block Jacobi beside the plain one, same Newton iterations;
    # the chosen method also runs to the end of the solve (time to solution)
    chosen = None
    if not mixed and args.chosen:
        from intpointsfem_gb300 import train_preconditioner as tp

        def mixed_arm(learned_prec, to_end):
            C_ = ip.ElastoPlasticIntPointsStructMatrix(wb)
            if args.no_row_stencils:
                C_.set_row_stencils(0)
            C_.set_precision(ip.MIXED)
            set_inner(C_)
            if learned_prec:
                C_.set_node_grid(2 * n + 1, 2 * n + 1)
                C_.mlp_init(0)
                C_.set_mlp_params(tp.load_weights())
                C_.set_preconditioner(ip.PREC_MLP)
            elif not args.jacobi:
                C_.set_preconditioner(ip.PREC_BLOCK_JACOBI)
            uc = torch.zeros(C_.neq, dtype=torch.float64, device=dev)
            sc_ = torch.cuda.ExternalStream(C_.stream, device=dev)
            C_.newton_begin(N_STEPS, newton_max_it=40, cg_rtol=args.mixed_cg_rtol)
            pw = timed_advance(C_, sc_, uc, args.warmup, e0, e1)
            l0c = C_.launch_count
            stc, msc = timed_advance(C_, sc_, uc, args.steps, e0, e1)
            nc = max(1, stc.newton_iters)
            out = {"ms_per_newton_iter": msc / nc,
                   "cg_iters_per_newton": stc.cg_iters / max(1, stc.newton_iters),
                   "newton_iters_timed": stc.newton_iters, "fcg_fallbacks": stc.fcg_fallbacks,
                   "ms_cg_per_newton": stc.ms_solve / nc, "gpu_launches": C_.launch_count - l0c}
            if to_end:
                pr = timed_advance(C_, sc_, uc, 0, e0, e1)
                out["solve"] = solve_record([pw, (stc, msc), pr], N_STEPS)
            if not learned_prec:
                out["ms_spmv_fp32"] = C_.profile_spmv(reps=20)
                # the FP32 strain gather and residual scatter (the FP32 residual option)
                C_.set_residual_precision(32)
                out["residual_kernels_fp32"] = residual_kernel_roofline(
                    C_, C_.profile_residual(uc, 32), 4, measured_peaks()[0])
            C_.close()
            return out

        chosen = mixed_arm(True, args.solve)
        inner = (("adaptive inner tolerance (Eisenstat-Walker, first solve of a step to %g)" % args.mixed_cg_rtol)
                 if args.inner == "adaptive" else "inner tolerance %g" % args.mixed_cg_rtol)
        if args.predictor == "on":
            inner += ", secant predictor of the load steps"
        if args.tangent == "consistent":
            inner += ", consistent spectral tangent"
        if args.spectral == "plane":
            inner += ", closed-form plane-strain spectral decomposition"
        chosen["method"] = ("mixed + learned: FP32 tangent, flexible CG preconditioned by the learned "
                            "triangular factor (weights shipped in intpointsfem_gb300/weights), %s, FP64 residual/"
                            "return mapping/Newton refinement" % inner)
        chosen["mixed_jacobi"] = mixed_arm(False, False)
        chosen["mixed_jacobi"]["method"] = "mixed: FP32 tangent + FP32 %s, %s, FP64 Newton refinement" % (
            "Jacobi-CG" if args.jacobi else "block-Jacobi CG", inner)
        chosen["speedup_vs_plain"] = ms_dev / chosen["ms_per_newton_iter"]
        chosen["note"] = ("the chosen method's Newton iterations are not the plain method's (secant predictor, "
                          "inexact inner solves, consistent tangent): its per-iteration ratio compares different "
                          "work; the time to solution (solve_speedup_vs_plain) is the like-for-like comparison")
        if solve_plain and "solve" in chosen:
            chosen["solve_speedup_vs_plain"] = solve_plain["ms"] / chosen["solve"]["ms"]

    # roofline of the dominant kernel (CG block SpMV), CUDA events on the library stream
    ms_spmv = A.profile_spmv(reps=20)
    # the residual kernels at the last Newton iterate, CUDA events between them
    res_bits = 32 if (mixed and args.residual32) else 64
    res_kernels = residual_kernel_roofline(A, A.profile_residual(du, res_bits), res_bits // 8, measured_peaks()[0])
    nb, nn = A.n_blocks, A.n_nodes
    nb_stored, _, upper_only = A.layout_info(fp32=mixed)      # the FP32 tangent may hold the upper blocks only
    vb = 16 if mixed else 32                                   # bytes of one 2x2 block
    stencils = A.row_stencil_count()[1 if mixed else 0] > 0 and not args.no_row_stencils
    # 8-bit stencil id per row (and a transposed-stencil id with the upper-only layout), or a column per block
    idx_bytes = nn * (2 if upper_only else 1) if stencils else 4 * nb_stored
    spmv_bytes = nb_stored * vb + idx_bytes + nn * (vb + 4 + 2)  # blocks, indices; p read, q write, rowlen, fixed
    hbm_peak, peak_kind = measured_peaks()
    achieved = spmv_bytes / (ms_spmv * 1e-3) / 1e9
    spmv_fp64_tflops = 2.0 * (4 * nb + 2 * nn) / (ms_spmv * 1e-3) / 1e12

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        arm = CpuArm(n, args.cpu_threads or os.cpu_count(), args.n_steps, args.wb, block=not args.jacobi)
        cpu = arm.sample(cg_per_iter, args.cpu_cg_sample)
        arm.close()

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    cfg = workload_config(args)
    if mixed:
        cfg["workload"] = cfg["workload"].replace("plain FP64", "mixed FP32/FP64").replace(
            "CG 1e-8", ("CG adaptive (first solve %g)" if args.inner == "adaptive" else "CG %g") % cg_rtol)
        cfg["cg_rtol"] = cg_rtol
        cfg["inner_tolerance"] = args.inner
    cfg["replicas"] = ws
    line = {
        "metric": METRIC, "value": ms_dev, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_dev, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if not mixed else "f32+f64", "data": "synthetic",
        "config": cfg,
        "row_stencils": bool(stencils),
        "ip_per_s": A.n_ip / (ms_res * 1e-3),
        "ms_residual": ms_res,
        "residual_kernels": res_kernels,
        "cg_iters_per_newton": cg_per_iter,
        "newton_iters_timed": st.newton_iters,
        "ms_breakdown": {"assemble": st.ms_assemble / n_timed, "cg": st.ms_solve / n_timed,
                         "commit": st.ms_commit / n_timed},
        "e2e": ({"value": ms_e2e, "unit": UNIT, "h2d_bytes_per_step": 8 * A.neq, "d2h_bytes_per_step": 8 * A.neq,
                 "how": "one ipfem_newton_advance(u, 1, IPFEM_HOST) call per step: u (8 B x neq) copied H2D "
                        "and D2H inside every timed step"}
                if ms_e2e is not None else None),
        "precision": args.precision,
        "roofline": {"kernel": "k_cg_spmv_sym" if upper_only else "k_cg_spmv", "bound": "hbm",
                     "achieved": achieved, "peak": hbm_peak,
                     "unit": "GB/s", "frac": achieved / hbm_peak, "peak_kind": peak_kind,
                     "traffic": SPMV_DRAM_BYTES[bool(stencils)] if (n == 400 and not mixed) else None,
                     "algorithmic_bytes": spmv_bytes,
                     "ms_per_launch": ms_spmv,
                     "layout": {"stored_blocks": nb_stored, "upper_only": upper_only}},
        "gpu_launches": launches,
    }
    if not mixed:                                              # the FP64 SpMV also meets the FP64 pipe's roofline
        line["roofline"]["fp64"] = {"achieved_tflops": spmv_fp64_tflops, "peak_tflops": fp64_tflops,
                                    "frac": spmv_fp64_tflops / fp64_tflops,
                                    "peak_kind": "measured live (fma probe)"}
    if solve_plain:
        line["solve"] = solve_plain
    if chosen:
        line["chosen"] = chosen
    if clk:
        line["clocks"] = clk
    if cpu:
        line["cpu_baseline"] = {"value": cpu["ms_per_newton"], "unit": UNIT, "cores": args.cpu_threads or os.cpu_count(),
                                "kind": "port",
                                "sample": "C oracle (bit-identical arithmetic): one tangent assembly (%.0f ms) + %d "
                                          "CG iterations (%.2f ms each), scaled by the %.0f CG iterations per "
                                          "Newton iteration measured here on the GPU; residual %.1f ms = %.3g IP/s"
                                          % (cpu["t_asm_ms"], cpu["cg_sample"], cpu["t_cg_iter_ms"], cg_per_iter,
                                             cpu["t_res_ms"], cpu["ip_per_s"])}
    print(json.dumps(line))
    sys.stdout.flush()
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ipfem", choices=["ipfem", "reference"])
    ap.add_argument("--config", type=int, default=2, choices=sorted(CONFIGS))
    ap.add_argument("--n", type=int, default=0, help="mesh size (default: the configuration's)")
    ap.add_argument("--cpu-threads", type=int, default=0)
    ap.add_argument("--cpu-cg-sample", type=int, default=100)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision", default="plain", choices=["plain", "mixed"])
    ap.add_argument("--mixed-cg-rtol", type=float, default=None,
                    help="inner FP32 tolerance of the mixed methods: of the first solve of a load step with the "
                         "adaptive inner tolerance (default 3e-2), of every solve with --inner fixed (default 3e-3)")
    ap.add_argument("--inner", default="adaptive", choices=["adaptive", "fixed"],
                    help="inner tolerance of the mixed methods' Newton iterations")
    ap.add_argument("--predictor", default="on", choices=["on", "off"],
                    help="secant predictor at the start of each load step of the mixed methods (the chosen "
                         "method's setting: on)")
    ap.add_argument("--tangent", default="consistent", choices=["consistent", "reference"],
                    help="tangent of the mixed methods: the consistent spectral tangent (the chosen method's "
                         "setting) or the reference's TangentOperator; the plain method keeps the reference's")
    ap.add_argument("--spectral", default="reference", choices=["reference", "plane"],
                    help="spectral decomposition of the mixed methods: the reference's (default) or the closed form "
                         "of plane-strain tensors (ipfem_set_spectral_mode); the plain method keeps the reference's")
    ap.add_argument("--no-chosen", dest="chosen", action="store_false")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--residual32", action="store_true",
                    help="with --precision mixed: FP32 strain gather and residual scatter (FP64 refinement)")
    ap.add_argument("--no-solve", dest="solve", action="store_false",
                    help="skip the time to solution (the rest of the solve after the timed iterations)")
    ap.add_argument("--jacobi", action="store_true", help="scalar Jacobi instead of block Jacobi in the CG")
    ap.add_argument("--no-row-stencils", action="store_true",
                    help="SpMVs read the stored column indices instead of the row stencils (same results)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    cfg = CONFIGS[args.config]
    args.n = args.n or cfg["n"]
    args.n_steps = cfg["n_steps"]
    args.wb = dict(cfg["wb"])
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
