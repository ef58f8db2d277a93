"""Command line front end in the reference's formats.

Reads instance files as the reference's solvers do (width*width
whitespace-separated tiles per file, e.g. benchmarks/yama24_50_hard_new/probNNN,
read by input_table at src/24puzzle_block_parallel_with_pdb.cu:433-452), prints
one `<file> <len> <nodes>` line per instance (the line format of
src/24puzzle_expand_with_pdb.cpp:284-285 and of benchmarks/pdb_expand_nodes.csv)
and optionally writes the reference's timing CSV: one seconds value per line
(src/24puzzle_block_parallel_with_pdb.cu:963), which test/calculate_executed_sum.cpp
sums.

    python sliding-puzzle_gb300/slide_cli.py --width 5 --heuristic pdb \\
        --csv result.csv ../benchmarks/yama24_50_hard_new/prob*

By default all instances are solved as one batch and each CSV line holds the
batch's wall time divided by the number of instances (so the CSV sums to the
batch's wall time); --one-by-one solves them one call at a time, as the
reference does, and writes each call's wall time.
"""
import argparse
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def read_instance(path, width):
    """The tiles of one instance file (whitespace-separated integers)."""
    with open(path) as f:
        vals = [int(x) for x in f.read().split()]
    n = width * width
    if len(vals) < n:
        raise ValueError("%s: %d values, %d expected" % (path, len(vals), n))
    t = np.array(vals[:n], dtype=np.int64)
    if sorted(t.tolist()) != list(range(n)):
        raise ValueError("%s: not a permutation of 0..%d" % (path, n - 1))
    return t.astype(np.uint8)


def format_line(name, result):
    return "%s %d %d" % (name, result["len"], result["nodes_total"])


def write_csv(path, seconds):
    with open(path, "w") as f:
        for s in seconds:
            f.write("%f\n" % s)


def run(solver, paths, one_by_one=False, clock=time.perf_counter):
    """(lines, seconds per instance) for the instance files `paths`."""
    tiles = np.stack([read_instance(p, solver.width) for p in paths]) if paths else \
        np.zeros((0, solver.width * solver.width), np.uint8)
    names = [os.path.basename(p) for p in paths]
    if one_by_one:
        results, secs = [], []
        for t in tiles:
            t0 = clock()
            results.append(solver.solve(t[None])[0])
            secs.append(clock() - t0)
    else:
        t0 = clock()
        results = solver.solve(tiles)
        wall = clock() - t0
        secs = [wall / max(1, len(paths))] * len(paths)
    for r, p in zip(results, paths):
        if r["status"] != 0:
            raise RuntimeError("%s: status %d" % (p, r["status"]))
    return [format_line(n, r) for n, r in zip(names, results)], secs


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("files", nargs="+")
    ap.add_argument("--width", type=int, choices=(4, 5), default=5)
    ap.add_argument("--heuristic", choices=("manhattan", "pdb"), default="pdb")
    ap.add_argument("--csv", default="")
    ap.add_argument("--one-by-one", action="store_true")
    a = ap.parse_args(argv)
    import slide
    with slide.Solver(a.width, a.heuristic) as s:
        if a.heuristic == "pdb":
            s.build_pdb()
        lines, secs = run(s, a.files, a.one_by_one)
    for line in lines:
        print(line)
    if a.csv:
        write_csv(a.csv, secs)


if __name__ == "__main__":
    main()
