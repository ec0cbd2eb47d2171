"""bench.py's reference arm on the CPU: one JSON line with the keys the measurement contract asks
for (the GPU arm needs a GPU and is exercised by the GPU runs)."""

import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_prints_one_contract_line():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    # a 20x8x8 box keeps the CPU run short; the line's layout does not depend on the size
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
                        "--warmup", "1", "--nx", "20", "--ny", "8", "--nz", "8"], capture_output=True, text=True,
                       cwd=ROOT, env=env, timeout=600)  # fmt: skip
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):  # fmt: skip
        assert k in d, k
    assert d["steps"] == 2 and d["warmup"] == 1 and d["value"] > 0 and d["higher_is_better"] is False
    assert d["config"]["workload"].startswith("hex8 J2 box 20x8x8")
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    # the value is extrapolated from measured parts and says so; ms_per_step is the sample's own wall time
    assert d["extrapolated"] is True and cb["extrapolated"] is True
    assert d["steps"] * d["ms_per_step"] / 1e3 <= d["wall_s"]
    parts = cb["newton_per_step"] * (cb["element_loop_s"] + cb["csr_update_s"] + cb["krylov_per_solve"] * cb["cg_iteration_s"])
    assert abs(parts - d["value"]) <= 1e-9 * d["value"]
    assert cb["krylov_per_solve"] > 0
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
