"""The bench's reference arm on the CPU: `bench.py --impl reference` times
the FP64 CPU oracle on the same workload and prints the contract's JSON line,
without building or loading the CUDA library (the scenario comes from the
oracle's generator twins; a reduced case here)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = """
import sys
sys.argv = ["bench.py", "--impl", "reference", "--small", "--steps", "1", "--warmup", "3"]
import bench
bench.main()
maps = open("/proc/self/maps").read()
print("PRODUCT_LIB_LOADED" if "libweldform_gb300" in maps else "PRODUCT_LIB_NOT_LOADED")
"""


def test_reference_arm_line_without_the_product_library():
    r = subprocess.run([sys.executable, "-c", PROBE], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = r.stdout.strip().splitlines()
    line = json.loads([ln for ln in lines if ln.startswith("{")][-1])
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["unit"] == "particle-steps/s"
    assert line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["config"]["preload_steps"] == 0
    assert "PRODUCT_LIB_NOT_LOADED" in lines
