"""bench.py --impl reference: the reference arm times the C oracle on the
reference's own W/E grids over a num_el-weighted sample of the benchmark
workload, names the GPU arm's config, and loads nothing of the library under
test (no `mcd` package, no libmcd.so)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r'''
import contextlib, io, json, sys
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"]
sys.path.insert(0, ".")
import bench
buf = io.StringIO()
with contextlib.redirect_stdout(buf):
    bench.main()
maps = open("/proc/self/maps").read()
print(json.dumps({"line": json.loads(buf.getvalue().strip().splitlines()[-1]),
                  "mcd_modules": sorted(m for m in sys.modules if m == "mcd" or m.startswith("mcd.")),
                  "libmcd_loaded": "libmcd.so" in maps, "oracle_loaded": "libmcd_oracle" in maps,
                  "config": bench.bench_config(bench.workload())}))
'''


def test_reference_arm_is_oracle_only_and_names_the_gpu_config():
    r = subprocess.run([sys.executable, "-c", PROBE], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    line = out["line"]
    assert line["impl"] == "reference" and line["metric"] == "scatter events/s" and line["value"] > 0
    assert line["config"] == out["config"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert out["mcd_modules"] == [] and not out["libmcd_loaded"] and out["oracle_loaded"]
    # the sample is weighted like the workload: about 40 000 electrons, every simulation present
    assert "num_el-weighted sample" in line["cpu_baseline"]["sample"]
    assert "electrons over the 64 sims" in line["cpu_baseline"]["sample"]
