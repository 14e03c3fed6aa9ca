"""The timeline summary of the diagnostic build's kernel records (host logic only)."""
import numpy as np

from picgo_gb300 import timeline


def write_records(path, recs):
    a = np.array([(s, e, (k << 32) | b) for s, e, k, b in recs], dtype=np.uint64)
    a.tofile(path)


def test_launch_grouping_and_busy_time(tmp_path):
    p = tmp_path / "t.bin"
    # fil_energy_bulk (6): two blocks of one launch, overlapping; then a second launch 5 us later.
    # exvol (17) runs beside the first launch; a finalizer section (22) lies inside fin_energy (5).
    write_records(p, [
        (1_000, 11_000, 6, 0), (1_200, 10_500, 6, 1),
        (2_000, 6_000, 17, 0),
        (12_000, 15_000, 5, 0), (12_100, 13_000, 22, 0),
        (20_000, 30_000, 6, 0),
    ])
    t0, t1, kid, blk = timeline.load(str(p))
    L = timeline.launches(t0, t1, kid)
    assert [(k, a, b, n) for k, a, b, n in L if k == 6] == [(6, 1_000, 11_000, 2), (6, 20_000, 30_000, 1)]
    text = timeline.summarize(str(p), iterations=2)
    first = text.splitlines()[0]
    assert "launches 4" in first                      # sections are not launches
    assert "wall 29.0 us" in first and "busy 23.0 us" in first
    assert "fin_energy: loads" in text
    assert "wall per iteration 14.5 us" in text
