"""Run the reference's own serial solvers (compiled by ref_build.sh into
oracle/_ref/bin) on arbitrary instances -- TEST INFRASTRUCTURE.

The reference programs read hard-coded relative paths
(src/24puzzle_expand.cc:183 `../benchmarks/yama24_50_med/probNNN`,
src/24puzzle_expand_with_pdb.cpp:78-79 `../pdb/pat24.*.tab`, :308
`../benchmarks/yama24_50_hard_new/probNNN`) and write `../result/*.csv`.
This module lays out oracle/_ref/run/{benchmarks,pdb,result,cwd} so those
paths resolve, writes the instances (padding the fixed instance count with
goal states), runs the binary with cwd=run/cwd and parses `path len nodes`.
"""
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BIN = os.path.join(HERE, "_ref", "bin")
RUN = os.path.join(HERE, "_ref", "run")


def _layout(folder, states, count, width):
    base = os.path.join(RUN, "benchmarks", folder)
    shutil.rmtree(base, ignore_errors=True)
    os.makedirs(base)
    os.makedirs(os.path.join(RUN, "result"), exist_ok=True)
    os.makedirs(os.path.join(RUN, "cwd"), exist_ok=True)
    goal = np.arange(width * width)
    for i in range(count):
        s = states[i] if i < len(states) else goal
        with open(os.path.join(base, "prob%03d" % i), "w") as f:
            f.write(" ".join(str(int(x)) for x in s) + "\n")


def _run(binary, n, timeout=3600):
    out = subprocess.run([os.path.join(BIN, binary)], cwd=os.path.join(RUN, "cwd"), capture_output=True,
                         text=True, timeout=timeout).stdout
    rows = []
    for line in out.splitlines():
        p = line.replace("pdb is installed.", "").split()
        p = [x for x in p if x.startswith("../benchmarks") or x.lstrip("-").isdigit()]
        if len(p) >= 3 and p[0].startswith("../benchmarks"):
            rows.append((int(p[1]), int(p[2])))
    return rows[:n]


def run_md24_expand(states):
    """src/24puzzle_expand.cc on up to 51 instances: [(len, nodes mod 2^32)]."""
    _layout("yama24_50_med", states, 51, 5)
    return _run("24puzzle_expand", len(states))


def write_tab_files(tables):
    """Write oracle tables as the reference's pat24.*.tab files (compact rank
    order is exactly the byte order its loader reads)."""
    d = os.path.join(RUN, "pdb")
    os.makedirs(d, exist_ok=True)
    for name, t in zip(("pat24.1256712.tab", "pat24.34891314.tab"), tables):
        p = os.path.join(d, name)
        if not (os.path.exists(p) and os.path.getsize(p) == t.size):
            t.tofile(p)


def run_pdb24_expand(states, tables):
    """src/24puzzle_expand_with_pdb.cpp on up to 50 instances: [(len, nodes)]."""
    write_tab_files(tables)
    _layout("yama24_50_hard_new", states, 50, 5)
    return _run("24puzzle_expand_with_pdb", len(states))
