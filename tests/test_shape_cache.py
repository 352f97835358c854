"""The tuned-shape cache file without a GPU: gs_load_shape_cache reads the tuner's JSON
format, skips entries with invalid shapes, and refuses a missing file."""
import pytest


def test_load_shape_cache(gs, tmp_path):
    path = tmp_path / "shapes.json"
    good = ('{"device": "NVIDIA GB300", "sms": 152, "algorithm": 1, "box_mode": 1, "key_bits": 12, "math": 0, '
            '"flags": 368, "n_bucket": 18, "sort_keys_per_thread": 8, "sort_lookback": 32, "scan_lookback": 64, '
            '"force_warps": 2, "force_short_lists": 0, "direct_targets": 2, "direct_blocks_per_sm": 12, '
            '"moment_blocks_per_sm": 2, "best_ms": 0.4, "default_ms": 0.45}')
    bad = good.replace('"force_warps": 2', '"force_warps": 3')  # no such kernel
    path.write_text('{"format": "gsim-shapes-1", "entries": [\n' + good + ",\n" + bad + "\n]}\n")
    gs.clear_shape_table()
    assert gs.load_shape_cache(str(path)) == 1
    gs.clear_shape_table()
    with pytest.raises(gs.GsimError):
        gs.load_shape_cache(str(tmp_path / "missing.json"))
