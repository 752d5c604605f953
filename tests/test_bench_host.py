"""The bench's host-side pieces, without a GPU: the DRAM traffic it reports beside the
roofline comes from the committed ncu summary of the stage-2 kernel on the bench
workload, and both arms label the same workload."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def test_traffic_per_cell_is_read_from_the_stage2_profile():
    import bench
    v = bench.read_traffic()
    assert v is not None, f"no traffic_bytes_per_cell line in {bench.TRAFFIC_PROFILE}"
    # stage 2 reads 11 and writes 5 values per member-cell (64 B in float32) and also
    # reads back the stage-1 planes that miss L2: between the algorithmic 64 B and 64 + 24 B
    assert 64.0 <= v <= 88.0, v


def test_both_arms_name_the_same_workload():
    import bench
    cfg = bench.workload_config(64)
    assert cfg["members"] == 64 and cfg["cells_per_step"] == 64 * 400 * 325
    assert cfg["grid"] == "400x325" and "batched uniform" in cfg["workload"]
