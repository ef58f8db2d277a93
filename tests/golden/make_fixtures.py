"""Regenerate the golden fixtures in this folder from the reference checkout.

Run in a container where the reference checkout is mounted:

    python tests/golden/make_fixtures.py REFERENCE_ROOT
    SLIDE_REFERENCE_DIR=REFERENCE_ROOT python tests/golden/make_fixtures.py

It copies, as JSON, the reference's own instance files and golden answers:
  korf100.json          benchmarks/korf100/probNNN + test/result_15puzzle.txt
  yama24_hard_new.json  benchmarks/yama24_50_hard_new/probNNN
                        + benchmarks/manhattan_expand_nodes.csv
                        + benchmarks/pdb_expand_nodes.csv
  yama24_med.json       benchmarks/yama24_50_med/probNNN
                        + test/result_24puzzle.txt lines 52-153
  yama24_50.json        benchmarks/yama24_50/probNNN + test/result_24puzzle.txt lines 1-51
and the fingerprints of the oracle-built pattern databases:
  pdb_fingerprints.json sha256 and value histogram of every table
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def read_instance(path):
    with open(path) as f:
        return [int(x) for x in f.read().split()]


def golden_rows(path):
    rows = {}
    with open(path) as f:
        for line in f:
            p = line.split()
            if len(p) >= 2:
                rows[os.path.basename(p[0])] = [int(x) for x in p[1:]]
    return rows


def main(ref):
    bench = os.path.join(ref, "benchmarks")
    # korf100: 15-puzzle, optimal lengths
    k = golden_rows(os.path.join(ref, "test", "result_15puzzle.txt"))
    korf = [{"name": "prob%03d" % i, "tiles": read_instance(os.path.join(bench, "korf100", "prob%03d" % i)),
             "len": k["prob%03d" % i][0]} for i in range(100)]
    json.dump({"source": "benchmarks/korf100, test/result_15puzzle.txt", "width": 4, "instances": korf},
              open(os.path.join(HERE, "korf100.json"), "w"), indent=0)
    # yama24_50_hard_new: all-solutions node counts, Manhattan and PDB
    md = golden_rows(os.path.join(bench, "manhattan_expand_nodes.csv"))
    pdb = golden_rows(os.path.join(bench, "pdb_expand_nodes.csv"))
    hard = [{"name": "prob%03d" % i,
             "tiles": read_instance(os.path.join(bench, "yama24_50_hard_new", "prob%03d" % i)),
             "md": md["prob%03d" % i], "pdb": pdb["prob%03d" % i]} for i in range(50)]
    json.dump({"source": "benchmarks/yama24_50_hard_new, benchmarks/{manhattan,pdb}_expand_nodes.csv",
               "width": 5, "instances": hard}, open(os.path.join(HERE, "yama24_hard_new.json"), "w"), indent=0)
    # yama24_50_med: first-solution counts (PDB lines 52-102, Manhattan 103-153)
    lines = open(os.path.join(ref, "test", "result_24puzzle.txt")).read().splitlines()
    pdb_first = {os.path.basename(l.split()[0]): [int(x) for x in l.split()[1:]] for l in lines[51:102]}
    md_first = {os.path.basename(l.split()[0]): [int(x) for x in l.split()[1:]] for l in lines[102:153]}
    med = [{"name": "prob%03d" % i,
            "tiles": read_instance(os.path.join(bench, "yama24_50_med", "prob%03d" % i)),
            "pdb_first": pdb_first["prob%03d" % i], "md_first": md_first["prob%03d" % i]} for i in range(51)]
    json.dump({"source": "benchmarks/yama24_50_med, test/result_24puzzle.txt:52-153", "width": 5,
               "instances": med}, open(os.path.join(HERE, "yama24_med.json"), "w"), indent=0)
    y50 = {os.path.basename(l.split()[0]): int(l.split()[1]) for l in lines[0:51]}
    inst50 = [{"name": "prob%03d" % i, "tiles": read_instance(os.path.join(bench, "yama24_50", "prob%03d" % i)),
               "len": y50["prob%03d" % i]} for i in range(51)]
    json.dump({"source": "benchmarks/yama24_50, test/result_24puzzle.txt:1-51", "width": 5, "instances": inst50},
              open(os.path.join(HERE, "yama24_50.json"), "w"), indent=0)
    # oracle pattern-database fingerprints
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import numpy as np
    import oracle
    fp = {}
    for w in (4, 5):
        for t, arr in enumerate(oracle.tables(w)):
            fp["%d_%d" % (w, t)] = {"sha256": hashlib.sha256(arr.tobytes()).hexdigest(), "size": int(arr.size),
                                    "hist": np.bincount(arr, minlength=int(arr.max()) + 1).tolist()}
    json.dump({"source": "oracle/pdb_oracle.c, ORC_PDB_BLANK_HOME", "tables": fp},
              open(os.path.join(HERE, "pdb_fingerprints.json"), "w"), indent=1)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SLIDE_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: make_fixtures.py REFERENCE_ROOT (or set SLIDE_REFERENCE_DIR)")
    main(ref)
