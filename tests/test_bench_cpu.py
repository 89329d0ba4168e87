"""bench.py's bookkeeping (no GPU): which force form a call takes, how many
kernels it launches and how many FP64 instructions it executes, mirroring
abie_gb300/csrc/force.cu; and the clock record read from nvidia-smi."""
import numpy as np

import bench
from abie_gb300 import ics


def test_force_form_selection():
    p, v, m, r = ics.planetesimal_disk()
    assert bench.force_path(m) == "sym"
    assert bench.launches_per_force_call(m) == 6
    m2 = m.copy()
    m2[5] = 0.0                      # one massless body: the chunked form
    assert bench.force_path(m2) == "chunked"
    assert bench.launches_per_force_call(m2) == 4
    p, v, m, r = ics.planetary_system()
    assert bench.force_path(m) == "queue" and bench.launches_per_force_call(m) == 2


def test_symmetric_instruction_count():
    p, v, m, r = ics.planetesimal_disk()
    inter = bench.interactions(m)
    per = bench.fp64_instructions_per_call(m, inter) / inter
    assert 4.5 < per < 4.55          # 9 per pair, plus the one-sided diagonal tiles
    m2 = m.copy()
    m2[5] = 0.0
    inter2 = bench.interactions(m2)
    assert bench.fp64_instructions_per_call(m2, inter2) == 6 * inter2


def test_clock_record_parsing(tmp_path):
    """The clock record reads nvidia-smi's CSV: median SM clock, the largest
    max clock, every throttle reason seen Active, the sample count."""
    import bench

    class _Done:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    rows = [
        "0, 2070, 2070, 250.5, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 2040, 2070, 260.1, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 1980, 2070, 262.0, 0x40, Not Active, Active, Not Active, Not Active",
        "garbage line",
    ]
    path = tmp_path / "clocks.csv"
    path.write_text("\n".join(rows) + "\n")
    c = bench.Clocks(0)
    c.proc, c.path = _Done(), str(path)
    rec = c.stop()
    assert rec["sm_mhz"] == 2040.0 and rec["sm_max_mhz"] == 2070.0
    assert rec["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    assert rec["samples"] == 3 and rec["power_w_max"] == 262.0


def test_energy_error_statistics():
    """The long-horizon runs' |dE/E| summary: percentiles, the count within
    1e-12, and against a reference distribution the systems within 10x of
    the reference's value for the same system."""
    de = np.array([1e-13, 5e-13, 2e-12, 1e-9])
    ref = np.array([2e-13, 1e-13, 1e-12, 1e-11])
    out = bench._de_stats(de, ref)
    assert out["systems"] == 4 and out["systems_at_or_below_1e-12"] == 2
    assert out["abs_dE_over_E_p50_p90_p99_max"][3] == 1e-9
    assert out["reference_method_at_or_below_1e-12"] == 3
    assert out["systems_within_10x_of_reference"] == 3   # 1e-9 > 10 x 1e-11
    q = out["reference_method_p50_p90_p99_max"]
    assert q[0] == np.percentile(ref, 50) and q[3] == 1e-11
