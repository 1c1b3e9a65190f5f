"""CPU tests of the kernel configuration table: defaults, validation,
save/load round trip (no device needed)."""
import os

import pytest

from preclib_gb300 import native


@pytest.fixture(autouse=True)
def _reset():
    native.tune_reset()
    yield
    native.tune_reset()


def test_defaults():
    d = native.tune_get(22)
    assert (d["log2_cols"], d["col_group"], d["col_radix_cap"], d["split_primes"]) == (11, 8, 6, 1)
    assert d["row_radix_cap"] == 4
    assert native.tune_get(20)["row_radix_cap"] == 6  # 2^10-point rows
    assert d["rows_per_cta"] == 1 and d["ms"] == 0.0
    d = native.tune_get(24)  # prime set 1: rows of 2^13
    assert d["log2_cols"] == 11
    d = native.tune_get(26)
    assert (d["log2_cols"], d["col_group"]) == (13, 4)
    assert native.tune_get(13)["split_primes"] == 0


@pytest.mark.parametrize("bad", [dict(log2_n=12, log2_cols=6, col_group=8, col_radix_cap=6, row_radix_cap=4, rows_per_cta=1),
                                 dict(log2_n=22, log2_cols=12, col_group=8, col_radix_cap=6, row_radix_cap=4, rows_per_cta=1),
                                 dict(log2_n=22, log2_cols=11, col_group=6, col_radix_cap=6, row_radix_cap=4, rows_per_cta=1),
                                 dict(log2_n=22, log2_cols=11, col_group=8, col_radix_cap=5, row_radix_cap=4, rows_per_cta=1),
                                 dict(log2_n=22, log2_cols=11, col_group=8, col_radix_cap=6, row_radix_cap=4, rows_per_cta=3),
                                 dict(log2_n=22, log2_cols=11, col_group=8, col_radix_cap=6, row_radix_cap=4, rows_per_cta=8),
                                 dict(log2_n=26, log2_cols=13, col_group=8, col_radix_cap=6, row_radix_cap=4, rows_per_cta=1),
                                 dict(log2_n=24, log2_cols=12, col_group=4, col_radix_cap=6, row_radix_cap=4, rows_per_cta=1),
                                 dict(log2_n=22, log2_cols=11, col_group=8, col_radix_cap=6, row_radix_cap=5, rows_per_cta=1)])
def test_invalid_configs_rejected(bad):
    with pytest.raises(native.PrecGpuError) as e:
        native.tune_set(**bad)
    assert e.value.code == native.E_ARG


def test_save_load_round_trip(tmp_path):
    native.tune_set(log2_n=20, log2_cols=9, col_group=4, col_radix_cap=4, row_radix_cap=4, rows_per_cta=2, split_primes=0, ms=0.07)
    native.tune_set(log2_n=22, log2_cols=11, col_group=8, col_radix_cap=4, row_radix_cap=4, rows_per_cta=4, split_primes=1)
    path = str(tmp_path / "tune.txt")
    native.tune_save(path)
    native.tune_reset()
    assert native.tune_get(20)["log2_cols"] == 10
    native.tune_load(path)
    t = native.tune_get(20)
    assert (t["log2_cols"], t["col_group"], t["col_radix_cap"], t["rows_per_cta"], t["split_primes"]) == (9, 4, 4, 2, 0)
    assert t["row_radix_cap"] == 4
    assert abs(t["ms"] - 0.07) < 1e-6
    assert native.tune_get(22)["rows_per_cta"] == 4


def test_load_rejects_bad_files(tmp_path):
    native.tune_set(log2_n=20, log2_cols=9, col_group=4, col_radix_cap=4, row_radix_cap=4, rows_per_cta=2, split_primes=0)
    bad = tmp_path / "bad.txt"
    bad.write_text("# prec_gpu tune 2\n20 10 8 6 6 1 1 0 0\n21 10 8 6 4 3 1 0 0\n")
    with pytest.raises(native.PrecGpuError):
        native.tune_load(str(bad))
    assert native.tune_get(20)["log2_cols"] == 9  # nothing installed
    nohdr = tmp_path / "nohdr.txt"
    nohdr.write_text("20 10 8 6 6 1 1 0 0\n")
    with pytest.raises(native.PrecGpuError):
        native.tune_load(str(nohdr))
    with pytest.raises(native.PrecGpuError):
        native.tune_load(os.path.join(str(tmp_path), "missing.txt"))
