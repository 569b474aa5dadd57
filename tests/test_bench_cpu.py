"""bench.py's contract on the CPU: the reference arm's JSON line (rank 0,
a small N) and the size of the headline's summaries, which must keep the
last stdout line to a few KB whatever the suites hold."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_line():
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                        "--n", "1024", "--steps", "2", "--warmup", "1"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["cpu_baseline"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] in ("port", "reference")
    assert line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["config"]["n"] == 1024


def _case(**extra):
    c = {"ms_per_fcompute": 2.123456789, "bodies_per_s": 493712345.6789, "p50": 0.00296628,
         "p99": 0.0104391973, "walk_node_gbs": 1134.19223, "interactions_per_body": 3142.11}
    c.update(extra)
    return c


def _suite():
    judge = {"step": 6, "p50_learned": 0.00708768842741847, "p99_learned": 0.0310686336830259,
             "p50_plain": 0.004696800373494625, "p99_plain": 0.023775570653378993,
             "rms_learned": 0.010808189184609933, "rms_plain": 0.007317517812162026,
             "used_plain": True, "samples": 4096, "judged_steps": 7, "fallback_steps": 7}
    best = {}
    for tgt in ("0.01", "0.001", "0.0001"):
        best[tgt] = {"best": {"path": "bh hilbert quadrupole lambda=3.9825", "lambda": 3.9825,
                              "ms": 16.389333605766296, "p99": 9.602686786350585e-05,
                              "p50": 2.3870617063260765e-05},
                     "bodies_per_s": 63979172.38264508,
                     "speedup_vs_reference_method": 14.274957514052849}
    bh = {"n": 1 << 20, "accuracy_frontier": {"best": best}}
    for k in ("hilbert_theta_0.5", "plain_theta_0.5", "hilbert_theta_0.9",
              "learned_walk_theta_0.9", "learned_coherent_walk_theta_0.9", "fp64_theta_0.5"):
        bh[k] = _case()
    bh["learned_theta_0.9"] = _case(judge=judge)
    for k in ("learned_0.9_vs_hilbert_theta_0.5", "learned_0.9_vs_plain_theta_0.5",
              "learned_walk_0.9_vs_hilbert_theta_0.5", "learned_walk_0.9_vs_plain_theta_0.5"):
        bh[k] = {"bodies_per_s_ratio": 0.0712712345, "p99_ratio": 1.0000123}
    bh["rkdp_theta_0.5"] = {"advises": 5, "aborted_at_call_budget": False, "fcompute_calls": 315,
                            "bodies_per_s": 328100000.123, "max_recursion": 8,
                            "error_threshold": 1e-6, "accepted_substeps": 40,
                            "max_accepted_error": 7.712e-07, "hit_recursion_cap": False}
    ens = {"system_steps_per_s": 73940.123, "accepted_fraction": 0.7523681640625,
           "ms_per_step": 27.7012345, "pairs_per_s": 3.004e12, "fp32_fraction": 0.74841234,
           "energy_drift_median": 1.626e-10, "energy_drift_max": 3.661e-08, "bodies": 4299629,
           "autotuner": {"best": {"ensemble.symmetric": 1, "ensemble.pairs_per_lane": 2,
                                  "ensemble.blocks_per_sm": 0},
                         "force_ms": {str(i): 4.0 for i in range(12)}}}
    return bh, ens


def test_headline_summaries_stay_compact():
    sys.path.insert(0, str(ROOT))
    bench = pytest.importorskip("bench")
    bh, ens = _suite()
    s_bh = bench.bh_summary(bh)
    s_ens = bench.ensemble_summary(ens)
    assert "p99_le_0.0001" in s_bh and "learned_theta_0.9" in s_bh
    assert "judge" in s_bh["learned_theta_0.9"]
    assert "autotuner" not in json.dumps(s_ens)  # the tuner's table stays in the suites file
    size = len(json.dumps(s_bh)) + len(json.dumps(s_ens))
    print(f"\nsummaries {size} bytes")
    assert size < 2000
