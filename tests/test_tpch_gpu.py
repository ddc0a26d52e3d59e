"""Q14 on the GPU from .tbl files: the star join's sums equal a direct
computation over the same synthetic rows."""
import pytest

from tpch_synth import q14_sums, write_tables

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n_lineitem", [1, 4000, 60000])
def test_q14_matches_rows(gj, cuda, tmp_path, n_lineitem):
    li, pa, cols = write_tables(tmp_path, n_part=2000, n_lineitem=n_lineitem, seed=n_lineitem + 3)
    (s_promo, s_all), rev = gj.tpch_q14(li, pa)
    want = q14_sums(cols)
    assert (s_promo, s_all) == want
    assert rev == pytest.approx(100.0 * want[0] / want[1] if want[1] else 0.0, rel=1e-12)


def test_q14_no_lineitems(gj, cuda, tmp_path):
    _, pa, _ = write_tables(tmp_path, n_part=100, n_lineitem=1)
    li = tmp_path / "empty_lineitem.tbl"
    li.write_text("")
    (s_promo, s_all), rev = gj.tpch_q14(str(li), pa)
    assert (s_promo, s_all) == (0, 0) and rev == 0.0
