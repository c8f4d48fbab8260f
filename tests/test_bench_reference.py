"""bench.py's reference arm on CPU: one JSON line with the benchmark's metric and configuration
(the CUDA arm's, adaptive sampling and f64 sums included, apart from the integrator's name),
`impl: reference`, a `cpu_baseline` describing the run and an `e2e` with no host-device bytes."""
import json
import subprocess
import sys
from pathlib import Path
from types import SimpleNamespace

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_prints_one_complete_json_line(oracle_lib):
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [x for x in out.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"]["workload"] == "many_spheres_1M_tris_hdri2048"
    import bench

    want = json.loads(json.dumps(bench.config(SimpleNamespace(integrator="wavefront", gpus=1))))
    assert {k: v for k, v in d["config"].items() if k != "integrator"} == \
        {k: v for k, v in want.items() if k != "integrator"}
    assert d["config"]["adaptive"] == {"threshold": 0.02, "min_spp": 16} and d["config"]["sums"] == "f64"
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
