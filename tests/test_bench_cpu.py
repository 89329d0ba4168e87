"""bench.py's bookkeeping of the force forms (no GPU): which form a call
takes, how many kernels it launches and how many FP64 instructions it
executes, mirroring abie_gb300/csrc/force.cu."""
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
