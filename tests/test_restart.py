"""Restart-tree files in the reference's layout and formats (restart.py):
raw big-endian FP64 arrays, the six Chebyshev bounds, and the Anderson
history list that drops its oldest entries."""
import numpy as np

from ttdft_public_gb300 import restart


def test_wfn_is_raw_big_endian_column_major(tmp_path):
    X = np.random.default_rng(0).standard_normal((7, 3))
    restart.write_wfn(str(tmp_path), (2, 3, 4), X)
    p = tmp_path / "rank_2_3_4" / "wfn" / "wfn_proc0"
    raw = p.read_bytes()
    assert len(raw) == 7 * 3 * 8
    assert np.array_equal(np.frombuffer(raw, ">f8"), X.ravel(order="F"))
    assert np.array_equal(restart.read_wfn(str(tmp_path), (2, 3, 4), 7, 3), X)


def test_bounds_round_trip_and_text_form(tmp_path):
    b = dict(zip(restart.BOUNDS, [12.5, 0.25, -3.0, 0.001, -0.2, -220.8185]))
    restart.write_bounds(str(tmp_path), (5, 5, 5), b)
    text = (tmp_path / "rank_5_5_5" / "wfn" / "cheby_bounds.txt").read_text()
    assert len(text.split("\t")) == 6 and "e+01" in text
    assert restart.read_bounds(str(tmp_path), (5, 5, 5)) == b


def test_history_keeps_the_newest_entries(tmp_path):
    root, r = str(tmp_path), (3, 3, 3)
    for it in range(6):
        f = {k: np.full(10, float(it)) for k in restart.KINDS}
        kept = restart.write_history_entry(root, r, it, f, keep=3)
    assert kept == [3, 4, 5] == restart.read_history(root, r)
    assert not (tmp_path / "rank_3_3_3" / "rho" / "rho_quad_in" / "rho_quad_in_scf2_proc0").exists()
    a = restart.read_array(restart.rho_file(root, r, "quad_out", 4), 10)
    assert np.all(a == 4.0)
