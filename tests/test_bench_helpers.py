"""Host-side helpers of bench.py: the timed window, the replayed L/M choices
and the SM-issue estimate built on per-unit instruction counts (no GPU)."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from swiftlink_gb300 import philox  # noqa: E402


def test_timed_window_starts_on_a_scoring_iteration():
    for W in (0, 1, 3, 5, 25):
        it0, itw = bench.window(W, 20)
        assert it0 % bench.PERIOD == 0 and it0 >= bench.PERIOD
        assert it0 - itw == W * bench.STEP_ITERS and itw >= 0


def test_lm_choices_replay_the_run():
    C, it0, it1, seed = 6, 100, 110, 5
    n_l = bench.lm_choices(C, it0, it1, seed, 0.5)
    want = [sum(philox.chooses_l(seed, c, it, 0.5) for c in range(C)) for it in range(it0, it1)]
    assert list(n_l) == want


def test_issue_estimate_counts_every_chain_iteration():
    C, it0, it1 = 10, 500, 700
    counts = {"l_half_sweep_per_chain": 1e5, "fag_per_meiosis_step": 2e3, "scan_per_meiosis_step": 1e3}
    r = bench.issue_estimate(C, it0, it1, bench.SEED, bench.LPROB, 184, 2070.0, 152, 1.0, counts)
    assert r["l_sweeps"] + r["m_sweeps"] == C * (it1 - it0)
    assert 0.4 < r["l_sweeps"] / (C * (it1 - it0)) < 0.6
    inst = r["l_sweeps"] * r["warp_inst_per_l_sweep"] + r["m_sweeps"] * r["warp_inst_per_m_sweep"]
    assert abs(r["achieved"] - inst / 1e9) < 1e-6 * r["achieved"]
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12
    assert r["warp_inst_per_m_sweep"] == 185 * 2e3 + 184 * 1e3
    assert bench.issue_estimate(C, it0, it1, bench.SEED, bench.LPROB, 184, None, 152, 1.0, counts) is None
    assert bench.issue_estimate(C, it0, it1, bench.SEED, bench.LPROB, 184, 2070.0, 152, 1.0, {}) is None


def test_issue_estimate_takes_the_lane_group_in_use():
    """The L-sampler's count is picked by the lane group the autotuner kept;
    a lane group without a count gives no estimate; with the classes' time
    shares each class's fraction uses its share of the time."""
    C, it0, it1 = 10, 500, 700
    counts = {"l_half_sweep_per_chain_by_lanes": {"32": 4e5, "8": 1e5}, "fag_per_meiosis_step": 2e3,
              "scan_per_meiosis_step": 1e3}
    r8 = bench.issue_estimate(C, it0, it1, bench.SEED, bench.LPROB, 184, 2070.0, 152, 1.0, counts, 8)
    r32 = bench.issue_estimate(C, it0, it1, bench.SEED, bench.LPROB, 184, 2070.0, 152, 1.0, counts, 32)
    assert r8["warp_inst_per_l_sweep"] == 2e5 and r32["warp_inst_per_l_sweep"] == 8e5
    assert bench.issue_estimate(C, it0, it1, bench.SEED, bench.LPROB, 184, 2070.0, 152, 1.0, counts, 16) is None
    r = bench.issue_estimate(C, it0, it1, bench.SEED, bench.LPROB, 184, 2070.0, 152, 1.0, counts, 8,
                             {"l": 0.25, "m": 0.75})
    peak = 152 * 4 * 2070.0e6
    assert abs(r["frac_l_sweeps"] - r["l_sweeps"] * 2e5 / (0.25 * peak)) < 1e-12
    assert abs(r["frac_m_sweeps"] - r["m_sweeps"] * r["warp_inst_per_m_sweep"] / (0.75 * peak)) < 1e-12


def test_per_iteration_cost_mixes_sweeps_and_scoring():
    t = {"lsweep_s": 2.0, "msweep_s": 6.0, "score_s": 100.0}
    assert abs(bench.per_iteration_s(t, 0.5) - (4.0 + 1.0)) < 1e-12


def test_counters_file_parses():
    c = bench.counters()
    assert isinstance(c, dict)
    assert np.all([isinstance(k, str) for k in c])
