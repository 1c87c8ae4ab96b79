"""The benchmark's reference arm on the CPU: one JSON line in the contract's
shape, timed on the oracle port of the reference's algorithm, with the product
library never mapped into the process (its bodies come from the oracle's IC
generator)."""
import json
import subprocess
import sys

import pytest

from conftest import ROOT

SCRIPT = r"""
import contextlib, io, json, sys
sys.argv = ["bench.py", "--impl", "reference", "--config", CONFIG, "--steps", "1",
            "--warmup", "3"]
import bench
buf = io.StringIO()
with contextlib.redirect_stdout(buf):
    bench.main()
maps = open("/proc/self/maps").read()
print(json.dumps({"line": buf.getvalue().strip().splitlines()[-1],
                  "product_mapped": "libcosmosim_gb300" in maps}))
"""


@pytest.mark.parametrize("config,n_bodies", [("disk20k", 20000), ("ensemble64", 1102884)])
def test_reference_arm_line_and_no_product_library(config, n_bodies):
    script = SCRIPT.replace("CONFIG", repr(config))
    r = subprocess.run([sys.executable, "-c", script], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["product_mapped"] is False
    line = json.loads(out["line"])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["steps"] == 1 and line["warmup"] == 3
    assert line["higher_is_better"] is True
    assert line["config"]["n_bodies"] == n_bodies
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["cpu_baseline"]["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
