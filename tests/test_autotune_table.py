"""The autotuner's table logic (no GPU): workload keys and the JSON table."""
import json

from orb_slam2_detailed_comments_gb300 import autotune


def test_workload_keys():
    assert autotune.workload_key([(640, 480)], 1000) == "640x480/1000"
    assert autotune.workload_key([(640, 480), (640, 480)], [1000, 1000]) == "640x480/1000"
    k = autotune.workload_key([(1280, 720), (640, 480), (1280, 720)], [2000, 1000, 2000])
    assert k == "batch:1280x720/2000,640x480/1000"


def test_table_round_trip_and_merge(tmp_path):
    p = str(tmp_path / "tuning.json")
    autotune.save_table({"640x480/1000": {"resize_rows": {"value": 16}}}, p)
    autotune.save_table({"knn": {"knn_tc_min_pairs": {"value": 123}}}, p)
    t = autotune.load_table(p)
    assert t["640x480/1000"]["resize_rows"]["value"] == 16
    assert t["knn"]["knn_tc_min_pairs"]["value"] == 123
    assert json.load(open(p)) == t


def test_parameters_are_the_library_names():
    assert set(autotune.PARAMS) == {"resize_rows", "fast_cells_per_block", "describe_group", "describe_depth"}
    for values, stage in autotune.PARAMS.values():
        assert stage in ("resize_blur", "fast", "describe") and len(values) >= 2


def test_small_launch_policies():
    assert set(autotune.POLICIES) == set(autotune.FULL_SIZE) == {"describe_task", "fast_chunk", "strip_rows_small"}
    assert autotune.POLICIES == {"describe_task": 0, "fast_chunk": 0, "strip_rows_small": 8}
    assert not set(autotune.POLICIES) & set(autotune.PARAMS)
