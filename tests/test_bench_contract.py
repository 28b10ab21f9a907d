"""The benchmark's contract on CPU: the reference arm (the CPU restatement on
the host cores) prints one JSON line with the keys the benchmark line
carries, and every per-tile figure the GPU arm reads from the committed ncu
summary is there and positive."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

FIGURES = ["traffic_bytes_per_tile_step", "canopy_warp_instructions_per_tile_step",
           "canopy_threads_per_warp_instruction", "soil_heat_fp64_warp_instructions_per_tile_step",
           "soil_water_fp64_warp_instructions_per_tile_step"]


def test_profile_figures_the_benchmark_reads():
    import bench
    for key in FIGURES:
        v = bench.profile_figure(key)
        assert v is not None and v > 0, key


def test_reference_arm_prints_one_contract_line():
    env = dict(os.environ, WORLD_SIZE="1", RANK="0", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--mp", "6000"], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-500:]
    lines = [ln for ln in r.stdout.strip().splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    b = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in b, k
    assert b["impl"] == "reference" and b["value"] > 0 and b["higher_is_better"] is True
    assert b["e2e"]["h2d_bytes_per_step"] == 0 and b["e2e"]["d2h_bytes_per_step"] == 0
    assert b["e2e"]["value"] == b["value"] and b["cpu_baseline"]["value"] == b["value"]
    assert b["cpu_baseline"]["kind"] == "port" and b["cpu_baseline"]["cores"] >= 1
    assert "workload" in b["config"]
