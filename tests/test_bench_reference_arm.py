"""bench.py's reference arm: the oracle on the bench's own mesh, on the host
cores, without loading any of the product package (CPU only)."""
import json
import os
import subprocess
import sys

from conftest import ROOT

PROBE = r"""
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--n", "24", "--steps", "2", "--warmup", "1"]
try:
    runpy.run_path("bench.py", run_name="__main__")
except SystemExit:
    pass
loaded = sorted(m for m in sys.modules if m.startswith("dgcuda_gb300"))
maps = open("/proc/self/maps").read() if sys.platform.startswith("linux") else ""
print("LOADED", loaded, "libdg_gb300" in maps)
"""


def test_reference_arm_loads_no_product_code(oracle_mod):
    r = subprocess.run([sys.executable, "-c", PROBE], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    line = json.loads(next(l for l in lines if l.startswith("{")))
    assert line["impl"] == "reference" and line["steps"] == 2
    assert line["config"]["elements"] == 2 * 24 * 24
    assert line["cpu_baseline"]["kind"] == "port" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert lines[-1] == "LOADED [] False"
