"""bench.py reads the walk's per-ray ncu figures from the committed profile summary (no GPU): the issue-side
roofline's warp instructions per ray and the DRAM bytes per ray of the bench step's capture, and the issue
activity and lanes per instruction of the persistent walk's bulk launch (bounce 1), not of the packet walk."""
import os
import re
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def profile_text():
    with open(os.path.join(ROOT, "profiles", "k_wf_extend_stress.md")) as f:
        return f.read()


def test_per_ray_figures_come_from_the_bench_step_capture():
    text = profile_text()
    step = text[text.index("## The bench step itself"):text.index("Packet-walk variants")]
    assert bench.ncu_warp_inst_per_ray() == float(re.search(r"warp_inst_per_ray = ([0-9.]+)", step).group(1))
    assert bench.ncu_traffic_per_ray() == float(re.search(r"dram_bytes_per_ray = ([0-9.]+)", step).group(1))
    assert 100 < bench.ncu_warp_inst_per_ray() < 1000 and 20 < bench.ncu_traffic_per_ray() < 1000


def test_issue_profile_is_the_persistent_walks():
    prof = bench.ncu_issue_profile()
    text = profile_text()
    bounce1 = text[text.index("## Bounce 1 (`--set full`"):]
    lanes = float(re.search(r"smsp__thread_inst_executed_per_inst_executed \| ([0-9.]+)", bounce1).group(1))
    assert prof["lanes_per_instruction"] == lanes < 20  # the packet walk runs near 30 lanes
    assert 0 < prof["issue_active"] <= 1 and 0 <= prof["dram_throughput"] <= 1
