"""The autotuner's cache (opflow_tune_*): host logic only, no device work.  Choices are read from a cache
file (last line of a key wins, comments skipped), malformed files are refused with the line number, and
clear / set_cache(None) return to an empty in-memory cache."""
import pytest

from opflow_gb300 import _capi as capi
from opflow_gb300 import api


@pytest.fixture
def fresh():
    api.tune_set_cache(None)
    api.tune_clear()
    yield
    api.tune_set_cache(None)
    api.tune_clear()


def test_cache_file_round_trip(fresh, tmp_path):
    p = tmp_path / "tune.txt"
    p.write_text("# opflow tuner\n"
                 "mg_smooth_z/f32/256x256x256/cell/1,1 8 0.0610\n"
                 "mg_tile/f32/2048x2048x1/cell/1,1 1 0.2000\n"
                 "mg_smooth_z/f32/256x256x256/cell/1,1 2 0.0590\n")
    api.tune_set_cache(p)
    assert api.tune_lookup("mg_smooth_z/f32/256x256x256/cell/1,1") == 2  # the last line of a key wins
    assert api.tune_lookup("mg_tile/f32/2048x2048x1/cell/1,1") == 1
    assert api.tune_lookup("axis3d/fixed/510x510x510/0") is None
    tuned, hits, entries = api.tune_stats()
    assert (tuned, hits, entries) == (0, 0, 2)
    api.tune_clear()
    assert api.tune_lookup("mg_tile/f32/2048x2048x1/cell/1,1") is None
    assert p.read_text().count("\n") == 4  # clearing keeps the file


def test_missing_file_is_an_empty_cache(fresh, tmp_path):
    api.tune_set_cache(tmp_path / "absent.txt")
    assert api.tune_stats()[2] == 0


def test_malformed_cache_is_refused(fresh, tmp_path):
    p = tmp_path / "bad.txt"
    p.write_text("mg_tile/f32/64x64x1/cell/1,1 1 0.1\nno-value-here\n")
    with pytest.raises(capi.OpflowError) as e:
        api.tune_set_cache(p)
    assert e.value.code == capi.E_INVALID and "line 2" in str(e.value)
