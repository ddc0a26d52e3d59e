"""TPC-H .tbl loader (host only): every Q14 column of synthetic tables, the
day numbers, and the errors for malformed rows, missing files and unsorted
part keys."""
import datetime

import numpy as np
import pytest

from tpch_synth import EPOCH, write_tables


def test_tpch_day(gj):
    for d in (datetime.date(1970, 1, 1), datetime.date(1992, 1, 1), datetime.date(1995, 9, 1),
              datetime.date(1995, 10, 1), datetime.date(2000, 2, 29), datetime.date(2098, 12, 31)):
        assert gj.tpch_day(d.year, d.month, d.day) == (d - EPOCH).days
    with pytest.raises(gj.GJError):
        gj.tpch_day(1995, 13, 1)


@pytest.mark.parametrize("n_lineitem", [1, 7, 4000])
def test_load_q14_columns(gj, tmp_path, n_lineitem):
    li, pa, cols = write_tables(tmp_path, n_lineitem=n_lineitem, seed=n_lineitem)
    got = gj.tpch_load_q14(li, pa)
    for name, want in cols.items():
        np.testing.assert_array_equal(got[name], want, err_msg=name)


def test_load_q14_errors(gj, tmp_path):
    li, pa, _ = write_tables(tmp_path, n_lineitem=50)
    with pytest.raises(gj.GJError):
        gj.tpch_load_q14(str(tmp_path / "missing.tbl"), pa)
    bad = tmp_path / "bad_lineitem.tbl"
    lines = open(li).read().splitlines(True)
    lines[20] = "1|2|3|\n"  # too few fields
    bad.write_text("".join(lines))
    with pytest.raises(gj.GJError, match="row 21"):
        gj.tpch_load_q14(str(bad), pa)
    unsorted = tmp_path / "unsorted_part.tbl"
    plines = open(pa).read().splitlines(True)
    plines[3], plines[4] = plines[4], plines[3]
    unsorted.write_text("".join(plines))
    with pytest.raises(gj.GJError):
        gj.tpch_load_q14(li, str(unsorted))


def test_load_q14_empty_files(gj, tmp_path):
    li, pa = tmp_path / "lineitem.tbl", tmp_path / "part.tbl"
    li.write_text("")
    pa.write_text("")
    got = gj.tpch_load_q14(str(li), str(pa))
    assert all(len(v) == 0 for v in got.values())
