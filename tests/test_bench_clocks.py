"""The bench's clock record (bench.py ClockSampler.summary, clocks_rejected):
nvidia-smi lines sampled during the timed region become the median SM clock,
the maximum clock and the active throttle reasons, and a record with a
hardware or thermal slowdown, or clocks held well below the maximum with no
reason, is rejected (the bench then times the region once more)."""
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
