"""CPU checks of bench.py's output contract: the reference arm's JSON line
(it runs the oracle on the host cores, no GPU needed), the silence of ranks
other than 0 under a multi-rank launch, and the roofline traffic figure."""
import argparse
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
SMALL = ["--tracks", "8", "--track-steps", "400", "--steps", "1", "--warmup", "1"]


def run_bench(extra, env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                           *extra], capture_output=True, text=True, timeout=300, env=env,
                          cwd=str(ROOT))


def test_reference_arm_prints_one_contract_line():
    r = run_bench(SMALL)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"] and cb["cores"] >= 1
    assert cb["kind"] in ("reference", "port") and cb["sample"]
    assert cb["model"]
    one = cb["single_core"]
    assert one["cores"] == 1 and one["value"] > 0 and one["unit"] == d["unit"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_print_nothing():
    r = run_bench(SMALL, {"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_roofline_traffic_is_the_full_launch_capture():
    """The traffic figure is the measured full-size launch, reported only for
    the run that capture describes (same tracks, steps, grid and seed)."""
    sys.path.insert(0, str(ROOT))
    import bench
    args = argparse.Namespace(track_steps=None, grid=None, seed=0)
    rd, wr, nt, sh, _ = bench.NCU_TRAFFIC["far"]
    shape = dict(zip(("points_per_lane", "lanes_per_direction", "steps_per_stage",
                      "track_subsets"), sh))
    t, src = bench.launch_traffic("far", args, nt, shape)
    assert t == rd + wr and "ncu" in src and "differs" not in src
    other_shape = dict(shape, track_subsets=sh[3] + 1)
    t, src = bench.launch_traffic("far", args, nt, other_shape)
    assert t == rd + wr and "differs" in src
    assert bench.launch_traffic("far", args, nt // 2, shape) == (None, None)
    assert bench.launch_traffic("ragged", args, nt, shape) == (None, None)
    for k, v in (("track_steps", 100), ("grid", [8, 8, 8]), ("seed", 3)):
        other = argparse.Namespace(**dict(vars(args), **{k: v}))
        assert bench.launch_traffic("far", other, nt, shape) == (None, None)
