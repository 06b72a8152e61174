"""bench.py's output contract where it runs without a GPU: the reference arm
(the CPU restatement of simple_astro timed on the host cores) prints one JSON
line with the metric and units of the GPU arm, a cpu_baseline describing the
run and an e2e object with no transfers; the argument parser keeps the
documented defaults."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "0", "--cpu-seconds", "0.3"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    import bench
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC
    assert d["unit"] == "Gpair-interactions/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1
    assert cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["config"] == bench.bench_config(bench.N_CUBE, 1)
    smp = d["sampling"]
    assert smp["total_rows"] == bench.N_CUBE + 4 and 0 < smp["rows_per_step"] <= smp["total_rows"]
    # ms_per_step is the time actually spent per sampled step, not an extrapolation
    assert abs(d["ms_per_step"] * d["steps"] / 1e3 - smp["seconds_timed"]) < 1e-6
    assert d["single_thread"]["cores"] == 1 and d["single_thread"]["value"] > 0


def test_reference_arm_leaves_the_cuda_library_unloaded():
    """The reference arm runs only the oracle: libphysim_gb300.so must not be
    mapped into its process (importing the package's numpy-only modules does
    not load it)."""
    code = ("import sys, bench; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', "
            "'--warmup', '0', '--cpu-seconds', '0.2']; bench.main(); "
            "import physim_gb300; maps = open('/proc/self/maps').read(); "
            "print('MAPPED', 'libphysim_gb300' in maps, physim_gb300.lib.loaded)")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                         timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    assert "MAPPED False False" in out.stdout, out.stdout[-500:]


def test_parser_defaults(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse()
    assert (a.gpus, a.impl, a.only) == (1, "ours", "")
    assert a.warmup >= 3 and a.steps >= 1
    assert a.serve_scheduling == "all" and a.serve_max_units == 2048
    assert a.serve_queue_ms == 0.0  # every idle unit ticked at once
    assert a.serve_seconds == 120.0  # the configured 120 s of arrivals
    assert a.bh_sample == 16384 and a.bh_steps == 1000


def test_parts_by_world_size():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.bench_parts("", 1) == ["direct", "bh", "ensemble", "served", "precision"]
    assert bench.bench_parts("", 8) == ["direct", "bh"]
    assert bench.bench_parts("served", 4) == ["served"]
