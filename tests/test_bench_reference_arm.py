"""bench.py --impl reference on the CPU: the reference's algorithm (the FP64
oracle) timed on the packed bed, printed as one JSON line with the keys the
benchmark contract names, without mapping the GPU library.  Under torchrun only
rank 0 runs it; the other ranks leave without work."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

_RUN = """
import sys
sys.path.insert(0, {root!r})
sys.argv = ["bench.py", "--impl", "reference", "--steps", "2", "--warmup", "3"]
import bench
bench.main()
maps = open("/proc/self/maps").read()
print("GPU_LIBRARY_MAPPED" if "libdem_gb300" in maps else "GPU_LIBRARY_NOT_MAPPED")
"""


def _run(env_extra=None):
    env = dict(os.environ, OMP_NUM_THREADS="4")
    env.pop("RANK", None)
    env.pop("WORLD_SIZE", None)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, "-c", _RUN.format(root=str(ROOT))], capture_output=True, text=True,
                          env=env, timeout=600)


def test_reference_arm_prints_the_contract_line_without_the_gpu_library():
    r = _run()
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["unit"] == "particle-steps/s" and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["value"] > 0 and abs(d["value"] - 200_000 / (d["ms_per_step"] * 1e-3)) <= 1e-6 * d["value"]
    assert d["config"]["workload"] == "wet200k-packed" and d["config"]["particles"] == 200_000
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "GPU_LIBRARY_NOT_MAPPED" in r.stdout


def test_reference_arm_runs_on_rank_zero_only():
    """a rank other than 0 exits 0 without timing or printing anything"""
    r = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1", "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": "29531"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")], r.stdout
