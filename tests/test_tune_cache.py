"""The contraction autotuner's cache file (falcon_set_tune_cache): its text
format is read back entry by entry, a file with another header or a
malformed line is refused, and decisions are appended to the file.  No GPU
is needed: the cache is host state (the measurements themselves are covered
by tests/test_gpu_tuning.py)."""
import pytest

HEADER = "falcon-contraction-tuning 2\n"


@pytest.fixture
def clean(fg):
    fg.tune_clear()
    yield
    fg.set_tune_cache(None)
    fg.tune_clear()


def test_cache_entries_read_back(fg, tmp_path, clean):
    f = tmp_path / "tune.txt"
    f.write_text(HEADER + "# comment lines and blank lines are skipped\n\n"
                 "NVIDIA_GB300_sm152 65 65 14 171 7 1 0 1 21.500 6.250 -1.000 30.000 25.000 -1.000\n"
                 "NVIDIA_GB300_sm152 65 65 43776 1 7 0 0 2 900.000 120.000 80.500 -1 -1 -1\n"
                 "NVIDIA_GB300_sm152 130 65 20 1 7 0 0 4 12.000 15.000 -1 13.000 11.000 12.500\n")
    fg.set_tune_cache(f)
    assert fg.tune_entries()[0] == 3
    path, us = fg.tune_lookup("NVIDIA_GB300_sm152", 65, 65, 14, 171, 7, 1, 0)
    assert path == "mma_sync" and us == {"fma": 21.5, "mma_sync": 6.25, "fma_ncol16": 30.0, "fma_ncol32": 25.0}
    path, us = fg.tune_lookup("NVIDIA_GB300_sm152", 130, 65, 20, 1, 7, 0, 0)
    assert path == "fma_ncol32" and us["fma_ncol64"] == 12.5
    path, us = fg.tune_lookup("NVIDIA_GB300_sm152", 65, 65, 43776, 1, 7, 0, 0)
    assert path == "tcgen05" and us["tcgen05"] == 80.5
    # another device, shape or reuse flag: no decision
    assert fg.tune_lookup("OTHER_sm10", 65, 65, 14, 171, 7, 1, 0) is None
    assert fg.tune_lookup("NVIDIA_GB300_sm152", 65, 65, 14, 171, 7, 1, 1) is None
    assert fg.tune_clear() == 3 and fg.tune_entries()[0] == 0


@pytest.mark.parametrize("body,what", [
    ("falcon-contraction-tuning 1\n", "header"),                                       # the old format
    (HEADER + "NVIDIA_GB300_sm152 65 65 14 171 7 1 0 6 1 1 1 1 1 1\n", "malformed line 2"),   # path 6
    (HEADER + "NVIDIA_GB300_sm152 65 65 0 171 7 1 0 1 1 1 1 1 1 1\n", "malformed line 2"),   # N = 0
    (HEADER + "NVIDIA_GB300_sm152 65 65 14 171 7 1 0 1 1 1 1\n", "malformed line 2"),         # 3 times
    (HEADER + "NVIDIA_GB300_sm152 65 65 14\n", "malformed line 2"),
])
def test_bad_cache_files_refused(fg, tmp_path, clean, body, what):
    f = tmp_path / "bad.txt"
    f.write_text(body)
    with pytest.raises(fg.FalconError, match=what):
        fg.set_tune_cache(f)


def test_missing_file_is_created_by_the_first_decision(fg, tmp_path, clean):
    # a path that does not exist yet is accepted (no decisions read)
    fg.set_tune_cache(tmp_path / "new.txt")
    assert fg.tune_entries()[0] == 0
    assert not (tmp_path / "new.txt").exists()
