"""bench.py's reference arm on the host cores: one JSON line with the keys the
bench contract names (a tiny case, so that it runs in the CPU suite)."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_prints_one_contract_line(oracle_mod):
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0",
                        "--n", "4096", "--cpu-sample", "256"],
                       cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, lines
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"]["workload"].startswith("plummer_disk") and d["config"]["n"] == 4096
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_tuner_table_names_are_distinct(gpu_lib):
    """Every autotuner candidate gets its own name in the bench line (a host
    lookup in the library; no device work)."""
    sys.path.insert(0, str(ROOT))
    import bench
    from physsim_gb300 import _native as N
    from physsim_gb300.system import BatchSystem
    names = [bench.tune_name(BatchSystem.tune_mode(m)) for m in range(N.BATCH_TUNE_MODES)]
    assert len(set(names)) == len(names), names
    assert "graph, grouped walk, 288-entry stack, 7 CTAs/SM" in names
