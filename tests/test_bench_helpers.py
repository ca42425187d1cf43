"""The benchmark's own bookkeeping without a GPU: the clock record parsed
from nvidia-smi samples (median SM clock, the throttle reasons a run is
judged by), the sort phase's algorithmic bytes for both key-table forms, the
peaks and ncu figures read from their committed files, and the rate of a
single replica."""
import json
import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


class _Done:
    """A finished sampler process."""

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def parsed(lines):
    import bench
    ck = bench.ClockSampler(0)
    ck.tmp.write("\n".join(lines) + "\n")
    ck.proc = _Done()
    return ck.stop()


def test_clock_record_median_and_reasons():
    # index, sm, max sm, power, active, hw_slowdown, hw_thermal, sw_thermal, sw_power_cap
    clean = ["0, 2070, 2070, 700.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"] * 3
    rec = parsed(clean + ["0, 1980, 2070, 900.0, 0x0000000000000004, Not Active, Not Active, "
                          "Not Active, Active"])
    assert rec["sm_mhz"] == 2070.0 and rec["sm_max_mhz"] == 2070.0
    assert rec["samples"] == 4
    assert rec["reasons"] == ["sw_power_cap"]  # kept and noted, not a rejection
    rec = parsed(clean + ["0, 1500, 2070, 1200.0, 0x08, Active, Not Active, Active, Not Active"])
    assert rec["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]
    # lines nvidia-smi could not fill are skipped; no sample at all gives None
    assert parsed(["0, [N/A], 2070, 1.0, 0x0, Not Active, Not Active, Not Active, Not Active"]) is None
    assert parsed([]) is None


def test_spatial_bytes_by_table_form():
    import bench
    n = 1 << 20
    # grid table: scan over its entries, scatter, reorder; no cell table
    assert bench.spatial_bytes(True, 1_800_000, n) == pytest.approx(12 * 1_800_000 / n + 120)
    # bucket table (n entries): the cell-table kernel's 40 B on top
    assert bench.spatial_bytes(False, n, n) == pytest.approx(12 + 120 + 40)


def test_committed_figures_are_read():
    import bench
    peak, kind = bench.peaks()
    if (ROOT / "MEASURED_PEAKS.json").exists():
        assert kind == "measured"
        want = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"]
        assert peak == pytest.approx(float(want))
    else:
        assert (peak, kind) == (6800.0, "fallback")
    d = json.loads((ROOT / "profiles" / "dram_traffic.json").read_text())
    for k in ("density", "pressure", "viscosity", "reorder"):
        assert bench.ncu_traffic("dam_break_1m", k) == d["dam_break_1m"][k]
    assert bench.ncu_traffic("dam_break_1m", "no_such_kernel") is None
    assert bench.ncu_issue("dam_break_1m", "density")["warp_inst_per_particle"] > 0


def test_single_replica_rate():
    import bench
    value, job_ms = bench.replica_throughput(1 << 20, 20, 13.3, 1, "cpu")
    assert job_ms == 13.3
    assert value == pytest.approx((1 << 20) * 20 / 0.0133)
