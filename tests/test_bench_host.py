"""The bench's host-side logic.

The clock record (bench.py ClockSampler.summary, clocks_rejected): nvidia-smi
lines sampled during the timed region become the median SM clock, the
maximum clock and the active throttle reasons, and a record with a hardware
or thermal slowdown, or clocks held well below the maximum with no reason,
is rejected (the bench then times the region once more).  The reference arm
(`--impl reference`, CPU only): its JSON line, and silence on ranks other
than 0."""
import bench


def record(lines):
    c = bench.ClockSampler(0)
    c.lines = lines
    return c.summary()


def line(sm, mx=2070, hw="Not Active", hwt="Not Active", swt="Not Active", cap="Not Active"):
    return f"0, {sm}, {mx}, 950.10, 0x0000000000000000, {hw}, {hwt}, {swt}, {cap}"


def test_summary_median_and_reasons():
    s = record([line(2070), line(2055), "garbage", "", line(1980, cap="Active"), "0, [N/A], 2070, 1, 0, a, b, c, d"])
    assert s["samples"] == 3 and s["sm_mhz"] == 2055 and s["sm_max_mhz"] == 2070
    assert s["reasons"] == ["sw_power_cap"]
    assert not bench.clocks_rejected(s)


def test_slowdowns_rejected():
    for kw in ({"hw": "Active"}, {"hwt": "Active"}, {"swt": "Active"}):
        s = record([line(2070), line(2070, **kw)])
        assert bench.clocks_rejected(s), kw


def test_low_clocks_without_reason_rejected():
    assert bench.clocks_rejected(record([line(1200)] * 5))            # a leftover clock lock
    assert not bench.clocks_rejected(record([line(1200, cap="Active")] * 5))  # power capped: kept
    assert not bench.clocks_rejected(record([line(1900)] * 5))
    assert not bench.clocks_rejected(record([]))                      # no nvidia-smi: nothing to judge


def _reference_arm(env_extra):
    import json
    import os
    import subprocess
    import sys
    env = dict(os.environ, **env_extra)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--config", "tiny", "--steps", "1",
                          "--warmup", "1", "--cpu-seconds", "1"], cwd=root, env=env, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    return [json.loads(l) for l in lines]


def test_reference_arm_line():
    """bench.py --impl reference (the oracle's integrator on the host cores)
    prints one line with the arm's contract keys, on the same metric and
    config keys as the GPU arm"""
    (line,) = _reference_arm({})
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == "paths/s"
    assert line["higher_is_better"] is True and line["value"] > 0 and line["steps"] == 1 and line["warmup"] == 1
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "paths/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["dataset"] == "tiny" and line["config"]["spp"] == 16


def test_reference_arm_other_ranks_silent():
    """under torchrun only rank 0 runs the reference arm; the others exit 0
    without a line"""
    assert _reference_arm({"RANK": "1", "WORLD_SIZE": "2"}) == []
