"""The launch-policy tuning table (tuning.cu): parsing, precedence of the
environment over the table, errors; and the committed table of the GB300
parses.  The table is process-wide state, so each test loads the table in
effect before it again at the end (an empty one if there was none)."""
import math
import os

import pytest

import network_relaxation_gb300 as nr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture
def lib(built, tmp_path):
    L = nr.lib()
    before = L.nr_tuning_source().decode()
    yield L
    if before:
        assert L.nr_tuning_load(before.encode()) >= 0
    else:
        empty = tmp_path / "empty.txt"
        empty.write_text("")
        assert L.nr_tuning_load(str(empty).encode()) == 0


def test_table_values_and_env_precedence(lib, tmp_path, monkeypatch):
    t = tmp_path / "t.txt"
    t.write_text("# comment\nNR_FP64_CLUSTER 8   # trailing comment\n\nNR_TILE_NODES 2048\n")
    monkeypatch.delenv("NR_FP64_CLUSTER", raising=False)
    monkeypatch.delenv("NR_TILE_NODES", raising=False)
    assert lib.nr_tuning_load(str(t).encode()) == 2
    assert lib.nr_tuning_value(b"NR_FP64_CLUSTER") == 8.0
    assert lib.nr_tuning_value(b"NR_TILE_NODES") == 2048.0
    assert math.isnan(lib.nr_tuning_value(b"NR_NOT_A_KNOB"))
    assert lib.nr_tuning_source().decode() == str(t)
    monkeypatch.setenv("NR_FP64_CLUSTER", "4")  # the environment overrides the table
    assert lib.nr_tuning_value(b"NR_FP64_CLUSTER") == 4.0


def test_table_errors(lib, tmp_path):
    assert lib.nr_tuning_load(str(tmp_path / "missing.txt").encode()) == nr.NR_ERR_IO
    for bad in ("NR_X\n", "NR_X 1 2\n", "lower_case 3\n"):
        p = tmp_path / "bad.txt"
        p.write_text(bad)
        assert lib.nr_tuning_load(str(p).encode()) == nr.NR_ERR_PARSE, bad


def test_committed_gb300_table_parses(lib):
    d = os.path.join(ROOT, "network_relaxation_gb300", "tuning")
    tables = [f for f in os.listdir(d) if f.endswith(".txt")] if os.path.isdir(d) else []
    if not tables:
        pytest.skip("no tuning table committed")
    for f in tables:
        n = lib.nr_tuning_load(os.path.join(d, f).encode())
        assert n > 0, f
        for name in ("NR_FP64_CLUSTER_NODES", "NR_TILE_MIN_NODES"):
            assert not math.isnan(lib.nr_tuning_value(name.encode())), (f, name)
