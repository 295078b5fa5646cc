"""The reference arm of bench.py (`--impl reference`) on the CPU: it times the oracle's path
tracer on a fixed row sample of the same workload, builds its scene from numpy and the oracle's
own triangulation, normals and intrinsics, and never loads the product library (libvgb.so)."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

_PROBE = r'''
import json, runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--scale", "0.04", "--steps", "1", "--warmup", "0"]
try:
    runpy.run_path("bench.py", run_name="__main__")
finally:
    maps = open("/proc/self/maps").read().splitlines()
    libs = sorted({l.split()[-1] for l in maps if l.split() and l.split()[-1].endswith(".so")})
    print("LIBS " + json.dumps(libs), file=sys.stderr)
'''


def test_reference_arm_runs_the_oracle_only():
    r = subprocess.run([sys.executable, "-c", _PROBE], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["config"]["workload"].startswith("path_traced")
    libs = json.loads([l for l in r.stderr.splitlines() if l.startswith("LIBS ")][-1][5:])
    assert any(p.endswith("libvgb_oracle.so") for p in libs)
    assert not any(Path(p).name == "libvgb.so" for p in libs), libs
