"""The benchmark's reference arm on the host cores: `bench.py --impl reference`
times the oracle (the CPU restatement of the reference's path) on a few rows
of the headline workload and prints one JSON line with the contract's keys.
The arm builds its inputs through the oracle library, so its process never
maps the CUDA library."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# runs bench.py as __main__ in this interpreter, then reports whether the
# process mapped the renderer's CUDA library
_RUNNER = r"""
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0", "--ref-rows", "8"]
runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print("LIBVRG_MAPPED" if "libvrg" in maps else "LIBVRG_NOT_MAPPED")
"""


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, "-c", _RUNNER], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert lines[-1] == "LIBVRG_NOT_MAPPED", lines[-1]
    line = json.loads(lines[-2])
    assert line["impl"] == "reference"
    assert line["metric"].startswith("Mrays/s and ms/frame @1080p ReSTIR")
    assert line["unit"] == "Mrays/s" and line["higher_is_better"] is True
    assert line["n_gpus"] == 1 and line["value"] > 0 and line["ms_per_step"] > 0
    assert line["config"]["workload"] == "restir-1080p-4x4chunks"
    assert line["config"]["resolution"] == [1920, 1080]
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
