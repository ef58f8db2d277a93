"""The command line front end's file handling on the CPU (a fake solver
stands in for the GPU): instance files in the reference's format, result
lines, and the one-seconds-value-per-line timing CSV."""
import numpy as np
import pytest

import slide_cli


class FakeSolver:
    width = 4

    def __init__(self):
        self.calls = 0

    def solve(self, tiles):
        self.calls += 1
        return [{"status": 0, "len": int(t[0]) + 10, "nodes_total": 1000 + int(t[1])} for t in tiles]


def _write(tmp_path, name, tiles, extra=""):
    p = tmp_path / name
    p.write_text(" ".join(str(int(x)) for x in tiles) + " " + extra + "\n")
    return str(p)


def test_reads_files_and_formats_lines(tmp_path):
    a = _write(tmp_path, "prob000", [1, 2, 3, 0, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15])
    b = _write(tmp_path, "prob001", np.arange(16)[::-1])
    t = iter([0.0, 0.5])
    lines, secs = slide_cli.run(FakeSolver(), [a, b], clock=lambda: next(t))
    assert lines == ["prob000 11 1002", "prob001 25 1014"]
    assert secs == [0.25, 0.25]  # the batch's wall time, split evenly


def test_one_by_one_times_each_call(tmp_path):
    a = _write(tmp_path, "p0", np.arange(16))
    b = _write(tmp_path, "p1", np.arange(16))
    t = iter([0.0, 1.0, 1.0, 3.0])
    s = FakeSolver()
    _, secs = slide_cli.run(s, [a, b], one_by_one=True, clock=lambda: next(t))
    assert s.calls == 2 and secs == [1.0, 2.0]


def test_rejects_bad_files(tmp_path):
    short = _write(tmp_path, "short", [1, 2, 3])
    dup = _write(tmp_path, "dup", [1] * 16)
    with pytest.raises(ValueError):
        slide_cli.read_instance(short, 4)
    with pytest.raises(ValueError):
        slide_cli.read_instance(dup, 4)


def test_csv_is_one_value_per_line(tmp_path):
    p = tmp_path / "out.csv"
    slide_cli.write_csv(str(p), [0.5, 1.25])
    vals = [float(x) for x in p.read_text().split()]
    assert vals == [0.5, 1.25] and p.read_text().count("\n") == 2
