"""Host-side helpers of bench.py (no GPU)."""

import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402


def test_spectral_power_db_error():
    rng = np.random.default_rng(5)
    t = np.linspace(-5, 5, 1024, endpoint=False)
    ref = np.exp(-t ** 2) * np.exp(1j * 0.3 * t ** 2)
    assert bench.spectral_power_db_error(ref, ref) == 0.0
    # a uniform 1% amplitude error is a 20 log10(1.01) dB power error everywhere
    assert abs(bench.spectral_power_db_error(1.01 * ref, ref) - 20 * np.log10(1.01)) < 1e-12
    # noise far below the -40 dB band does not count
    noisy = ref + 1e-9 * (rng.standard_normal(1024) + 1j * rng.standard_normal(1024))
    assert bench.spectral_power_db_error(noisy, ref) < 1e-3


def test_reference_arm_prints_the_contract_line():
    """``bench.py --impl reference`` on a short CPU sample: one JSON line with the keys of
    the benchmark line, the reference arm's cpu_baseline and an e2e without copies."""
    import json
    import subprocess

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ)
    env.pop("RANK", None)
    out = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "0", "--cpu-sample-s", "2"],
                         cwd=root, env=env, capture_output=True, text=True, timeout=600, check=True)
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 0
    assert d["n_gpus"] == 1 and d["ms_per_step"] > 0 and d["config"]["workload"] == bench.WORKLOAD
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == d["value"] and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
