"""bench.py's reference arm keeps the JSON-line contract on the host (no GPU):
the reference's CPU path (the oracle's OpenMP assembly) on the headline
workload, one line with the metric, its unit and the CPU-baseline record."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "assembled cells/s" and d["unit"] == "cells/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["n_gpus"] == 1 and d["steps"] == 1
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert "kuhn 3D 32^3" in d["config"]["workload"]


def test_device_arm_line_carries_every_contract_key():
    """The device arm's JSON line (built where it prints, checked here without a
    GPU by reading bench.py): every key of the bench contract, the roofline,
    CPU-baseline, end-to-end and clock records, and the workload name in config."""
    import ast

    tree = ast.parse(open(os.path.join(ROOT, "bench.py")).read())
    lines = [n.value for n in ast.walk(tree) if isinstance(n, ast.Assign) and isinstance(n.value, ast.Dict)
             and any(isinstance(t, ast.Name) and t.id == "line" for t in n.targets)
             and "roofline" in {k.value for k in n.value.keys if isinstance(k, ast.Constant)}]
    assert len(lines) == 1  # the device arm's line; the reference arm's is run above
    keys = {k.value for k in lines[0].keys if isinstance(k, ast.Constant)}
    for want in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                 "scaling", "vs_baseline", "dtype", "data", "config", "roofline", "e2e", "cpu_baseline",
                 "gpu_launches", "clocks", "parity"):
        assert want in keys, want
    config = lines[0].values[[k.value if isinstance(k, ast.Constant) else None for k in lines[0].keys].index("config")]
    assert "workload" in {k.value for k in config.keys if isinstance(k, ast.Constant)}
