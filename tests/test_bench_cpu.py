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
