"""bench.py's reference arm runs on the host alone: its JSON line keeps the
bench contract (metric, unit, config, cpu_baseline, e2e), and its Newton and
CG counts are the oracle's own, equal to a direct run of the same
iterations."""
import json
import os
import subprocess
import sys

import numpy as np

from oracle import pyoracle as po

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--n", "8", "--steps", "2",
                          "--warmup", "3", "--cpu-threads", "2"],
                         cwd=ROOT, capture_output=True, text=True, timeout=300, check=True)
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["dtype"] == "f64"
    assert line["steps"] == 2 and line["warmup"] == 3 and line["higher_is_better"] is False
    assert line["value"] > 0 and line["value"] == line["ms_per_step"] == line["e2e"]["value"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["config"]["mesh"] == "8x8" and line["config"]["load_steps"] == 20

    P = po.OracleProblem(po.default_params(8), nthreads=2)
    P.set_block_jacobi(True)
    u = np.zeros(P.neq)
    newton = po.OracleNewton(P, 20, newton_max_it=40, cg_rtol=1e-8)
    newton.advance(u, 3)
    k, cg = newton.advance(u, 2)
    P.close()
    assert line["newton_iters_timed"] == k == 2
    assert line["cg_iters_per_newton"] == cg / k


def test_clock_summary_from_nvidia_smi_lines():
    """The clock record of the bench line: median SM clock under the samples,
    the maximum, and every throttle reason seen Active (hw_slowdown,
    hw_thermal_slowdown and sw_thermal_slowdown reject a run, sw_power_cap is
    kept and noted); unparsable lines are skipped."""
    import bench

    class _Proc:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    idle = "Not Active"
    s = bench.ClockSampler(0)
    s.proc = _Proc()
    s.lines = ["2070, 2070, 812.4, 0x0000000000000000, %s, %s, %s, %s" % (idle, idle, idle, idle),
               "1965, 2070, 1391.0, 0x0000000000000004, %s, %s, %s, Active" % (idle, idle, idle),
               "2070, 2070, 1010.2, 0x0000000000000000, %s, %s, %s, %s" % (idle, idle, idle, idle),
               "[N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A]",
               "truncated, line"]
    rec = s.stop()
    assert rec == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    s2 = bench.ClockSampler(0)
    s2.proc = _Proc()
    s2.lines = ["1500, 2070, 700.0, 0x0000000000000008, Active, %s, %s, %s" % (idle, idle, idle)]
    assert s2.stop()["reasons"] == ["hw_slowdown"]
    s3 = bench.ClockSampler(0)
    assert s3.stop() is None


def test_residual_kernel_bytes_match_the_documented_per_point_figures():
    """The algorithmic bytes behind the residual kernels' roofline, for order-2
    elements at 400 x 400 (160 000 elements, 1 440 000 points, 641 601
    nodes): FP32 gather 99 B and scatter 92 B per point, FP64 gather 183 B
    per point (blocks 144, dofs 8, u 7.1 amortised, strains 24); achieved =
    bytes / time and frac = achieved / peak."""
    import types

    import bench

    n = 400
    M = types.SimpleNamespace(order=2, n_el=n * n, n_ip=9 * n * n, neq=2 * (2 * n + 1) ** 2,
                              n_colors=4, n_nodes=(2 * n + 1) ** 2)
    ms = {"gather_strain": 0.02, "stress_residual": 0.02, "color_reduce": 0.01, "compute_sigma": 1.0}
    r32 = bench.residual_kernel_roofline(M, ms, 4, 6797.2)
    r64 = bench.residual_kernel_roofline(M, ms, 8, 6797.2)
    per_point = lambda r, k: r[k]["algorithmic_bytes"] / M.n_ip  # noqa: E731
    assert round(per_point(r32, "gather_strain")) == 99
    assert round(per_point(r32, "stress_residual")) == 92
    assert round(per_point(r64, "gather_strain")) == 183
    g = r32["gather_strain"]
    assert abs(g["achieved_gbs"] - g["algorithmic_bytes"] / 0.02e-3 / 1e9) < 1e-9 * g["achieved_gbs"]
    assert abs(g["frac"] - g["achieved_gbs"] / 6797.2) < 1e-12
    assert r32["compute_sigma"] == {"ms": 1.0, "bound": "fp64 pipe"}
