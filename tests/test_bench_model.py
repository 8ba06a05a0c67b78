"""The work and byte models behind bench.py's roofline figures (no GPU)."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402


def test_fp64_instruction_model_degree4():
    # per cell-stage at degree 4: nodal, collocation, collocation with traces
    # (a last stage has one update FMA per DoF fewer); ncu counts about 4,000
    # FP64 instructions per cell for a traced stage
    assert bench.fp_work_per_cell(5)[0] == 8335
    assert bench.fp_work_per_cell(5, collocation=True)[0] == 4675
    assert bench.fp_work_per_cell(5, collocation=True, traces=True)[0] == 3925
    assert bench.fp_work_per_cell(5, stage=False, collocation=True, traces=True)[0] == 3925 - 125
    # upwind traces: one trace contraction per pencil and direction (3 x 25 x 5
    # FMAs fewer) and one product per face flux (2 x 75 fewer)
    assert bench.fp_work_per_cell(5, collocation=True, traces=True, upwind=True)[0] == 3925 - 375 - 150


def test_geometry_and_increment_bytes():
    assert bench.geometry_bytes_per_dof(5, 8) == 41.6
    assert abs(bench.geometry_bytes_per_dof(5, 4) - 20.8) < 1e-12
    # a 4-step block of the increment form: one FP64 anchor and 19 binary32 stages
    assert abs(bench.increment_bytes_per_dof_step(5) - 248.2) < 1e-9
    assert bench.bytes_per_dof_step() == 144
