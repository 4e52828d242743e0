"""Host-side helpers of bench.py: figures read from the committed ncu summaries
and the SM-issue estimate built on them (no GPU)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_instruction_counts_are_read_from_the_profiles():
    for name in ("sl_ls_jit_cfg2.md", "fag_warp_kernel_cfg2.md", "ffbs_scan_kernel_cfg2.md"):
        v = bench.inst_from_profiles(name)
        assert v is not None and v > 1e4, name
    assert bench.inst_from_profiles("no_such_profile.md") is None


def test_issue_estimate_counts_every_chain_iteration():
    C, it0, it1 = 10, 500, 700
    r = bench.issue_estimate(C, it0, it1, bench.SEED, bench.LPROB, 184, 2070.0, 152, 1.0)
    assert r["l_sweeps"] + r["m_sweeps"] == C * (it1 - it0)
    assert 0.4 < r["l_sweeps"] / (C * (it1 - it0)) < 0.6
    inst = r["l_sweeps"] * r["warp_inst_per_l_sweep"] + r["m_sweeps"] * r["warp_inst_per_m_sweep"]
    assert abs(r["achieved"] - inst / 1e9) < 1e-6 * r["achieved"]
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12
    assert bench.issue_estimate(C, it0, it1, bench.SEED, bench.LPROB, 184, None, 152, 1.0) is None
