"""The CPU legs of bench.py, run here on the host cores (no GPU): the headline's CPU baseline (the
oracle over the whole job), the miniapp loop bodies timed beside the GPU lines, and the
reference arm's JSON line. They run at the end of every GPU benchmark, so a failure here would cost
the whole line."""
import argparse
import contextlib
import io
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_cpu_baseline_and_miniapps():
    a = argparse.Namespace(cpu_steps=1)
    cb = bench.cpu_baseline(a, 64)
    assert cb["kind"] == "port" and cb["unit"] == "GB/s" and cb["value"] > 0 and cb["cores"] >= 1
    mini = bench.cpu_miniapps(iters=1)
    for k in ("stokes2d_1023_f64", "stokes3d_127_f64", "acoustic3d_255_f64"):
        assert mini[k]["ms"] > 0 and mini[k]["T_eff_GBs"] > 0
    assert mini["cores"] >= 1


@pytest.mark.parametrize("slab", [0, 16])
def test_reference_arm_line(slab):
    a = argparse.Namespace(n=64, ref_slab=slab, steps=1, warmup=0)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference(a, 1, 0)
    line = json.loads(buf.getvalue().strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == "T_eff" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
    # the default (slab 0) times the whole job, so the line names no sample
    assert ("z-slab" in line["config"]["workload"]) == (slab > 0)
