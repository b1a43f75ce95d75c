"""bench.py's host-side parts, without a GPU: the reference arm's JSON line
and the CPU samplers behind `cpu_baseline` and `configs`."""
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402
from linon_gb300 import workloads as wl  # noqa: E402
from oracle import pyoracle  # noqa: E402


def test_reference_arm_line():
    """--impl reference prints one JSON line with the contract's keys: the
    oracle port timed on the host cores, its e2e equal to its value."""
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0",
                        "--width", "96", "--height", "64"], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "ray-steps/s"
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"] == d["e2e"]["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["workload"].startswith("cornell_1920x1080")


def test_cpu_samplers():
    w = wl.plain_small(64, 48)
    v, threads, sample = bench.cpu_baseline(pyoracle, w, budget_s=0.2)
    assert v > 0 and threads >= 1 and "pixels" in sample
    views = wl.batch_views(3, seed=2, min_side=16, max_side=24)
    w.fields = [w.fields[0]] * 3
    v, threads, sample = bench.cpu_views_sample(pyoracle, views, w, budget_s=0.05)
    assert v > 0 and "rays" in sample and "views" in sample
    assert np.isfinite(v)


def test_flops_per_step_counts_live_operations():
    """The roofline's numerator: operations the endpoint depends on, per
    ray-step of the 1080p workload (h = 0.005, Kahan sums, field_weight 1).
    linear: f = v0 is loop-invariant, so only the Kahan sum of the position
    remains (4 operations x 3 components); twist: the y components of the
    field and of the stage positions are invariant; lens: every component
    is live; all below the count of every operation the oracle performs."""
    w = wl.frames_1080p()
    got = {name: bench.flops_per_step(pyoracle, w, wl._abi.FIELD_IDS[name]) for name in ("linear", "twist", "lens")}
    assert got["linear"] == (12.0, 0.0)
    assert got["twist"] == (57.0, 8.0)
    assert got["lens"] == (147.0, 4.0)
    e, f = np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32)
    pix = np.array([w.width // 2 + (w.height // 2) * w.width], np.int32)
    for name, (live, _) in got.items():
        ops, steps = pyoracle.count_ops(e, f, w.camera, w.settings, wl.fixed_steps(0.005, 64, kahan=True),
                                        wl._abi.FIELD_IDS[name], w.width, w.height, pix)
        assert live < ops[0, :4].sum() / steps[0]


class _Exited:
    """Stands in for the nvidia-smi process once its output was read."""

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def test_clock_sampler_keeps_the_timed_region():
    """Only samples that arrived inside the timed region count: the idle
    clock sampled before it starts does not lower the median, and a throttle
    reason seen afterwards is not reported; with no sample inside, every
    sample counts and the summary says so."""
    c = bench.ClockSampler(0)
    c.proc = _Exited()
    row = "{sm}, 2070, 900.0, Not Active, Not Active, Not Active, {cap}"
    c.lines = [(0.5, row.format(sm=1200, cap="Not Active")),
               (1.1, row.format(sm=2070, cap="Not Active")),
               (1.2, row.format(sm=2055, cap="Not Active")),
               (1.3, row.format(sm=2070, cap="Not Active")),
               (2.5, row.format(sm=1500, cap="Active"))]
    got = c.stop(1.0, 2.0)
    assert got["sm_mhz"] == 2070.0 and got["sm_max_mhz"] == 2070.0
    assert got["reasons"] == [] and got["samples"] == 3 and got["window"] == "timed region"
    c2 = bench.ClockSampler(0)
    c2.proc = _Exited()
    c2.lines = [(0.5, row.format(sm=2070, cap="Active"))]
    got = c2.stop(1.0, 2.0)
    assert got["samples"] == 1 and got["reasons"] == ["sw_power_cap"] and got["window"].startswith("whole")
