"""bench.py's reference arm (the oracle, the restatement of the reference's
loop nest, timed on the host cores) prints one JSON line with the keys,
units and types of the measurement contract and the same `config` as the
GPU arm; it needs no GPU and loads nothing of the engine."""
import json
import os
import subprocess
import sys

from conftest import ROOT

PROBE = """
import runpy, sys
sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'medium', '--steps', '1', '--warmup', '3']
runpy.run_path('bench.py', run_name='__main__')
mods = sorted(m for m in sys.modules if m == 'cipsi_gb300' or m.startswith('cipsi_gb300.'))
maps = open('/proc/self/maps').read()
print('ENGINE', mods, 'libcipsi_gb300' in maps)
"""


def test_reference_arm_prints_the_contract_line(oracle_exe):
    r = subprocess.run([sys.executable, "-c", PROBE], cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    line = [x for x in r.stdout.splitlines() if x.startswith("{")][-1]
    j = json.loads(line)
    assert j["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in j, k
    assert j["metric"] == "perturber contributions/s" and j["unit"] == "contributions/s"
    assert j["higher_is_better"] is True and j["n_gpus"] == 1 and j["steps"] == 1 and j["warmup"] >= 3
    assert j["value"] > 0 and j["ms_per_step"] > 0 and j["vs_baseline"] is None
    assert j["config"]["workload"].startswith("medium") and j["config"]["ncf"] == 2000
    cb = j["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == j["value"] and cb["sample"]
    assert j["e2e"] == {"value": j["value"], "unit": j["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # the reference arm neither imports nor loads the engine
    eng = [x for x in r.stdout.splitlines() if x.startswith("ENGINE")][-1]
    assert eng == "ENGINE [] False", eng
    # the GPU arm's config for the same workload is the same dict
    sys.path.insert(0, ROOT)
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    assert j["config"] == json.loads(json.dumps(bench.workload_desc("medium")))
    assert bench.workload_desc("large")["workload"].startswith("large") and bench.workload_desc("large")["ncf"] == 20000
