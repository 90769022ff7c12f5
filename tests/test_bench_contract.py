"""CPU tests of bench.py's reference arm (`--impl reference`), which the
benchmark contract runs beside the GPU arm: one JSON line with the same
metric, unit and config keys, a `cpu_baseline` describing the run, a
zero-copy `e2e`, and only the oracle library loaded in its process."""
import json
import os
import subprocess
import sys

from tests.conftest import ROOT

PROBE = r"""
import runpy, sys, json
sys.argv = ["bench.py", "--impl", "reference", "--steps", "2", "--warmup", "1",
            "--scene", "plain_16k"]
try:
    runpy.run_path("bench.py", run_name="__main__")
except SystemExit as e:
    assert not e.code, e.code
maps = open("/proc/self/maps").read()
print(json.dumps({"probe": True,
                  "product_so": "libpbf_gb300" in maps,
                  "product_py": "pbf_gb300._capi" in sys.modules,
                  "oracle_so": "liboracle" in maps or "pbf_oracle" in maps or "oracle/_build" in maps}))
"""


def test_reference_arm_line():
    env = dict(os.environ, OMP_NUM_THREADS="4")
    out = subprocess.run([sys.executable, "-c", PROBE], cwd=ROOT, env=env,
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [json.loads(l) for l in out.stdout.strip().splitlines() if l.startswith("{")]
    line, probe = lines[-2], lines[-1]
    assert probe["probe"] and probe["oracle_so"]
    assert not probe["product_so"] and not probe["product_py"]
    assert line["impl"] == "reference"
    assert line["metric"] == "particle-solver-iterations/s"
    assert line["unit"] == "particle-iters/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 2 and line["warmup"] == 1
    assert line["config"]["workload"] == "dam_break_16k"
    assert line["config"]["particles"] == 16384
    for k in ("grid", "dt", "window", "substeps_timed"):
        assert k in line["config"], k
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"],
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
