"""The autotuner's settings (ga_tune_*) without a GPU: defaults, range checks,
and the settings file (refused when malformed, nothing changed).  The GPU half
(every setting gives the same results; the search keeps its fastest
candidate) is in test_tune_gpu.py."""
import os

import pytest

from genoaligner_gb300 import api


def test_default_setting_is_valid_and_current_without_a_stored_one():
    d = api.tune_default()
    assert d == {"sw_pack16": 1, "sw_window": 2, "sw_long_log2": 24, "wfa_lane_smax": 31, "sw_coop_log2": 27,
                 "sw_opt16_pct": 100, "wfa_group": 16}
    if not api.device_available():
        assert api.tune_get() == d


@pytest.mark.parametrize("field,value", [("sw_pack16", 2), ("sw_window", 3), ("sw_window", 8),
                                         ("sw_long_log2", 15), ("sw_long_log2", 31),
                                         ("wfa_lane_smax", -1), ("wfa_lane_smax", 32),
                                         ("sw_coop_log2", 15), ("sw_coop_log2", 41),
                                         ("sw_opt16_pct", 49), ("sw_opt16_pct", 101),
                                         ("wfa_group", 4), ("wfa_group", 12), ("wfa_group", 64)])
def test_out_of_range_settings_are_refused(field, value):
    before = api.tune_get()
    with pytest.raises(ValueError):
        api.tune_set(**{field: value})
    assert api.tune_get() == before


def test_unknown_field_refused():
    with pytest.raises(ValueError):
        api.tune_set(tile=3)


@pytest.mark.parametrize("body", ["GB300\t1 2\n", "GB300 1 2 24 15 27 75\n", "GB300\t1 5 24 15 27 75\n",
                                  "GB300\tx y z w v u\n", "GB300\t1 2 24 15 27\n", "GB300\t1 2 24 15 27 30\n",
                                  "GB300\t1 2 24 15 27 100 12\n"])
def test_malformed_settings_file_refused(tmp_path, body):
    p = tmp_path / "tune.txt"
    p.write_text("# comment\n" + body)
    before = api.tune_get()
    with pytest.raises(ValueError):
        api.tune_load(str(p))
    assert api.tune_get() == before


def test_settings_file_roundtrip_without_device(tmp_path):
    p = tmp_path / "tune.txt"
    api.tune_save(str(p))                       # nothing stored: header only
    lines = [x for x in p.read_text().splitlines() if not x.startswith("#")]
    if not api.device_available():
        assert lines == []
    p.write_text("# ok\nSomeOtherGPU\t0 4 20 0 30 80\nOtherGPU2\t0 4 20 0 30 80 8\n")
    api.tune_load(str(p))                       # six or seven fields; other devices: nothing applied
    if not api.device_available():
        assert api.tune_get() == api.tune_default()


def test_missing_file_refused():
    with pytest.raises(ValueError):
        api.tune_load(os.path.join("/nonexistent-dir", "tune.txt"))
