"""Benchmark: ms per Newton iteration (and residual IP/s) of the plain FP64
wellbore solve, 400 x 400 order-2 quads (1.44 M integration points,
1 283 202 dofs), block-Jacobi CG to 1e-8 and Newton to 1e-8 relative
residual, on one GB300 (--jacobi: scalar Jacobi).

A step is one Newton iteration of the load-stepped solve (CG on the current
tangent, u += du, Assemble(K, rhs), convergence test; load-step acceptance
and the next step's first assembly fall inside the iteration where they
occur).  W warm-up iterations run untimed, then exactly K are timed.

  value    : device-timed (CUDA events on the library's stream), inputs resident
  e2e      : the same iterations through the C-ABI with pinned host buffers
             (u copied H2D and D2H every iteration), host-timed
  roofline : the CG block SpMV (dominant kernel), algorithmic bytes / launch
             over its CUDA-event duration, against the measured HBM copy peak
  cpu_baseline : the C oracle on the host cores, bounded sample (one tangent
             assembly + S CG iterations with the same preconditioner), scaled to
             a Newton iteration with the CG iteration count of the timed GPU
             iterations (the oracle performs bit-identical arithmetic, so the
             counts are the same)

--impl reference times the oracle alone (the reference's own CPU path cannot
be built: it needs NeoPZ, Intel MKL and TBB).
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
# CG iterations of the first Newton iterations of the 400 x 400 solve, as run on
# the GPU (identical on the CPU oracle), with block Jacobi and with Jacobi; used
# by --impl reference to scale its bounded CG sample to whole Newton iterations.
CFG2_CG_ITERS = [7001, 7822, 7021, 7695, 7021, 7913, 7021, 7895]
CFG2_CG_ITERS_JACOBI = [10119, 9495]
# DRAM bytes (read + write) of one FP64 SpMV launch at 400 x 400 (rows sorted
# by length), from the ncu captures summarised in profiles/k_cg_spmv_400x400.md:
# with row stencils, and with the stored column indices
SPMV_DRAM_BYTES = {True: 346.375424e6 + 4.631552e6, False: 388.405504e6 + 9.274112e6}
FALLBACK_HBM_GBS = 6800.0


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


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


def run_reference(args):
    ws, rank, _ = ddp_env()
    if rank != 0:
        return 0
    threads = args.cpu_threads or os.cpu_count()
    n = args.n
    arm = CpuArm(n, threads, args.n_steps, args.wb, block=not args.jacobi)
    if n <= 100:
        # small meshes: the oracle's own CG iteration count to 1e-8 on the first tangent
        R = arm.P.assemble(arm.u, 1.0 / args.n_steps)
        _, k = arm.P.pcg(R, rtol=1e-8, max_it=200000)
        cg_iters, cg_note = [abs(k)], "the oracle's CG iterations to 1e-8 on the first tangent"
    else:
        # the measured 400 x 400 counts, scaled by n / 400 (CG iterations grow linearly with n here)
        cg_iters = [c * n / 400.0 for c in (CFG2_CG_ITERS_JACOBI if args.jacobi else CFG2_CG_ITERS)]
        cg_note = "the GPU's CG iterations per Newton iteration at 400x400 scaled by n/400"
    mean_cg = sum(cg_iters) / len(cg_iters)
    samples = []
    for i in range(args.warmup + args.steps):
        cg = cg_iters[i] if i < len(cg_iters) else mean_cg
        r = arm.sample(cg, args.cpu_cg_sample if i >= args.warmup else 5)
        if i >= args.warmup:
            samples.append(r)
    arm.close()
    ms = statistics.mean(s["ms_per_newton"] for s in samples)
    line = {
        "impl": "reference", "metric": METRIC, "value": ms, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "wellbore %dx%d order-2 quads, %d IPs, plain FP64, %s 1e-8, Newton 1e-8, "
                               "%d load steps (configuration %d)"
                               % (n, n, 9 * n * n, "Jacobi-CG" if args.jacobi else "block-Jacobi CG", args.n_steps,
                                  args.config)},
        "ip_per_s": statistics.mean(s["ip_per_s"] for s in samples),
        "cpu_baseline": {"value": ms, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "per step: one tangent assembly + %d CG iterations of the C oracle, "
                                   "scaled to %.0f CG iterations per Newton iteration (%s)"
                                   % (samples[0]["cg_sample"], mean_cg, cg_note)},
        "e2e": {"value": ms, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


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
    cg_rtol = args.mixed_cg_rtol if mixed else 1e-8
    A = ip.ElastoPlasticIntPointsStructMatrix(wb)         # device-resident arm
    B = None if args.no_e2e else ip.ElastoPlasticIntPointsStructMatrix(wb)   # host-buffer (e2e) arm
    if mixed:
        A.set_precision(ip.MIXED)
        if B:
            B.set_precision(ip.MIXED)
    if not args.jacobi:
        A.set_preconditioner(ip.PREC_BLOCK_JACOBI)
        if B:
            B.set_preconditioner(ip.PREC_BLOCK_JACOBI)
    if args.no_row_stencils:
        A.set_row_stencils(0)
        if B:
            B.set_row_stencils(0)
    stream = torch.cuda.ExternalStream(A.stream, device=dev)
    fp64_tflops = A.measure_fp64_peak()

    # residual evaluation throughput (Assemble(rhs)), inputs resident
    du = torch.zeros(A.neq, dtype=torch.float64, device=dev)
    dr = torch.zeros_like(du)
    A.SetLoadFactor(1.0 / N_STEPS)
    for _ in range(3):
        A.assemble_residual(du, dr, ip.DEVICE)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nres = 20
    e0.record(stream)
    for _ in range(nres):
        A.assemble_residual(du, dr, ip.DEVICE)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_res = e0.elapsed_time(e1) / nres

    # Newton iterations, device-resident
    A.newton_begin(N_STEPS, newton_max_it=40, cg_rtol=cg_rtol)
    st_w, _ = A.newton_advance(du, args.warmup, ip.DEVICE)
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
    ms_dev = e0.elapsed_time(e1) / args.steps
    launches = A.launch_count - l0
    ms_dev = reduce_max(ms_dev, dist)
    cg_per_iter = st.cg_iters / max(1, st.newton_iters)

    # e2e through the C-ABI with pinned host buffers
    ms_e2e = None
    if B:
        hu = torch.zeros(B.neq, dtype=torch.float64, pin_memory=True)
        B.newton_begin(N_STEPS, newton_max_it=40, cg_rtol=cg_rtol)
        B.newton_advance(hu, args.warmup, ip.HOST)
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        B.newton_advance(hu, args.steps, ip.HOST)
        ms_e2e = 1e3 * (time.perf_counter() - t0) / args.steps
        B.close()

    # the chosen method (mixed precision + learned preconditioner) and mixed
    # precision with Jacobi beside the plain one, same Newton iterations
    chosen = None
    if not mixed and args.chosen:
        from intpointsfem_gb300 import train_preconditioner as tp

        def mixed_arm(learned_prec):
            C_ = ip.ElastoPlasticIntPointsStructMatrix(wb)
            if args.no_row_stencils:
                C_.set_row_stencils(0)
            C_.set_precision(ip.MIXED)
            if learned_prec:
                C_.set_node_grid(2 * n + 1, 2 * n + 1)
                C_.mlp_init(0)
                C_.set_mlp_params(tp.load_weights())
                C_.set_preconditioner(ip.PREC_MLP)
            elif not args.jacobi:
                C_.set_preconditioner(ip.PREC_BLOCK_JACOBI)
            uc = torch.zeros(C_.neq, dtype=torch.float64, device=dev)
            C_.newton_begin(N_STEPS, newton_max_it=40, cg_rtol=args.mixed_cg_rtol)
            C_.newton_advance(uc, args.warmup, ip.DEVICE)
            sc_ = torch.cuda.ExternalStream(C_.stream, device=dev)
            torch.cuda.synchronize()
            l0c = C_.launch_count
            e0.record(sc_)
            stc, _ = C_.newton_advance(uc, args.steps, ip.DEVICE)
            e1.record(sc_)
            torch.cuda.synchronize()
            out = {"ms_per_newton_iter": e0.elapsed_time(e1) / args.steps,
                   "cg_iters_per_newton": stc.cg_iters / max(1, stc.newton_iters),
                   "newton_iters_timed": stc.newton_iters, "fcg_fallbacks": stc.fcg_fallbacks,
                   "ms_cg_per_newton": stc.ms_solve / args.steps, "gpu_launches": C_.launch_count - l0c}
            if not learned_prec:
                out["ms_spmv_fp32"] = C_.profile_spmv(reps=20)
            C_.close()
            return out

        chosen = mixed_arm(True)
        chosen["method"] = ("mixed + learned: FP32 tangent, flexible CG to %g preconditioned by the learned "
                            "triangular factor (weights shipped in intpointsfem_gb300/weights), FP64 residual/"
                            "return mapping/Newton refinement" % args.mixed_cg_rtol)
        chosen["mixed_jacobi"] = mixed_arm(False)
        chosen["mixed_jacobi"]["method"] = "mixed: FP32 tangent + FP32 %s to %g, FP64 Newton refinement" % (
            "Jacobi-CG" if args.jacobi else "block-Jacobi CG", args.mixed_cg_rtol)
        chosen["speedup_vs_plain"] = ms_dev / chosen["ms_per_newton_iter"]

    # roofline of the dominant kernel (CG block SpMV), CUDA events on the library stream
    ms_spmv = A.profile_spmv(reps=20)
    nb, nn = A.n_blocks, A.n_nodes
    vb = 16 if mixed else 32                                   # bytes of one 2x2 block
    stencils = A.row_stencil_count()[1 if mixed else 0] > 0 and not args.no_row_stencils
    idx_bytes = nn if stencils else 4 * nb                     # 8-bit stencil id per row, or a column per block
    spmv_bytes = nb * vb + idx_bytes + nn * (vb + 4 + 2)       # blocks, indices; p read, q write, rowlen, fixed
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
    line = {
        "metric": METRIC, "value": ms_dev, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_dev, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64" if not mixed else "f32+f64",
        "data": "synthetic",
        "config": {"workload": "wellbore %dx%d order-2 quads, %d IPs, %d dofs, %s, %s %g, "
                               "Newton 1e-8, %d load steps%s; first %d Newton iterations (warm-up %d); "
                               "configuration %d"
                               % (n, n, A.n_ip, A.neq, "plain FP64" if not mixed else "mixed FP32/FP64",
                                  "Jacobi-CG" if args.jacobi else "block-Jacobi CG", cg_rtol,
                                  N_STEPS, (", material %s" % json.dumps(args.wb)) if args.wb else "",
                                  args.warmup + args.steps, args.warmup, args.config),
                   "l2": "inputs larger than L2 (tangent %.0f MB, element blocks %.0f MB)"
                         % (nb * 32 / 1e6, A.n_el * 1296 / 1e6),
                   "replicas": ws, "row_stencils": bool(stencils)},
        "ip_per_s": A.n_ip / (ms_res * 1e-3),
        "ms_residual": ms_res,
        "cg_iters_per_newton": cg_per_iter,
        "newton_iters_timed": st.newton_iters,
        "ms_breakdown": {"assemble": st.ms_assemble / args.steps, "cg": st.ms_solve / args.steps,
                         "commit": st.ms_commit / args.steps},
        "e2e": ({"value": ms_e2e, "unit": UNIT, "h2d_bytes_per_step": 8 * A.neq, "d2h_bytes_per_step": 8 * A.neq}
                if ms_e2e is not None else None),
        "precision": args.precision,
        "roofline": {"kernel": "k_cg_spmv", "bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                     "unit": "GB/s", "frac": achieved / hbm_peak, "peak_kind": peak_kind,
                     "traffic": SPMV_DRAM_BYTES[bool(stencils)] if (n == 400 and not mixed) else None,
                     "algorithmic_bytes": spmv_bytes,
                     "ms_per_launch": ms_spmv,
                     "fp64": {"achieved_tflops": spmv_fp64_tflops, "peak_tflops": fp64_tflops,
                              "frac": spmv_fp64_tflops / fp64_tflops, "peak_kind": "measured live (fma probe)"}},
        "gpu_launches": launches,
    }
    if chosen:
        line["chosen"] = chosen
    if clk:
        line["clocks"] = clk
    if cpu:
        line["cpu_baseline"] = {"value": cpu["ms_per_newton"], "unit": UNIT, "cores": args.cpu_threads or os.cpu_count(),
                                "kind": "port",
                                "sample": "C oracle (bit-identical arithmetic): one tangent assembly (%.0f ms) + %d "
                                          "CG iterations (%.2f ms each), scaled by %.0f CG iterations per "
                                          "Newton iteration; residual %.1f ms = %.3g IP/s"
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
    ap.add_argument("--mixed-cg-rtol", type=float, default=1e-4)
    ap.add_argument("--no-chosen", dest="chosen", action="store_false")
    ap.add_argument("--no-e2e", action="store_true")
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
