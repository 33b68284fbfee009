"""bench.py's reference arm on the CPU (the driver's `--impl reference`
launch): one JSON line with the contract's keys, the reference's own CPU path
(the oracle restatement) timed on a bounded sample."""
import json
import subprocess
import sys

import pytest

from conftest import ROOT


@pytest.mark.parametrize("config,unit", [("gps_l1_4mhz", "cells/s"), ("observables", "channel-epochs/s")])
def test_reference_arm_line(config, unit):
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--config", config,
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["unit"] == unit and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    if config == "gps_l1_4mhz":
        # the reference arm runs the oracle only, never the product library
        assert d["libraries_loaded"] and not any("libugsdr_cuda" in x for x in d["libraries_loaded"])
        assert d["anchor_full_search"]["extrapolated"] is False and d["single_thread"]["cores"] == 1
