"""CPU checks of bench.py's host helpers: the committed ncu summaries carry the per-launch
figures the bench line reports (DRAM traffic of the dominant kernels, the batched pass's
instruction count per group), so the roofline fields are never silently null."""
import os
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

import bench  # noqa: E402


def test_profiles_carry_the_bench_figures():
    t_batch = bench.profile_traffic("cand_batch_10Mx1024_b8.md")
    t_plain = bench.profile_traffic("cand_pass_10Mx1024_b8.md")
    ipg = bench.profile_number("cand_batch_10Mx1024_b8.md", "warp_instructions_per_group")
    # a 10M x 1024 8-bit launch reads about 491 MB of packets
    assert t_batch and 4.9e8 < t_batch < 6.0e8
    assert t_plain and 4.9e8 < t_plain < 6.0e8
    # about 22 instructions per group of four entries is the floor of the formulation
    assert ipg and 20 < ipg < 60
    assert bench.profile_number("cand_tc_2Mx1024_b4.md", "traffic_bytes_per_launch") > 2.5e9


def test_profile_number_missing_file_or_key():
    assert bench.profile_number("no_such_profile.md", "traffic_bytes_per_launch") is None
    assert bench.profile_number("cand_pass_10Mx1024_b8.md", "no_such_key") is None
