"""bench.py's reference arm (the reference's algorithm timed on the host cores) runs on the CPU
and prints the contract's JSON line; no device is used."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# runs bench.py in this interpreter, then reports whether the engine's library was ever mapped
RUN_AND_CHECK_MAPS = """
import runpy, sys
sys.argv = sys.argv[1:]
runpy.run_path(sys.argv[0], run_name="__main__")
maps = open("/proc/self/maps").read()
print("ENGINE_LIBRARY_MAPPED" if "libcntkmc" in maps else "ENGINE_LIBRARY_NOT_MAPPED", file=sys.stderr)
"""


@pytest.mark.parametrize("workload", ["cfg2", "cfg3", "cfg5"])
def test_reference_arm_prints_one_contract_line(workload):
    cmd = [sys.executable, "-c", RUN_AND_CHECK_MAPS, os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--workload", workload, "--steps", "1", "--warmup", "0", "--cpu-seconds", "1", "--films", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "hops/s" and d["value"] > 0
    for k in ("metric", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling", "vs_baseline",
              "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    assert d["config"]["workload"].startswith(workload)
    # the reference arm's inputs come from the oracle and numpy: the engine is never loaded
    assert "ENGINE_LIBRARY_NOT_MAPPED" in r.stderr


def test_gpu_arm_fails_loudly_without_a_device():
    # no CPU fallback: without a CUDA device the GPU arm exits non-zero and prints no bench line
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode != 0
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
