"""The CPU oracle against the reference's golden vectors (no GPU)."""
import hashlib
import os

import numpy as np
import pytest

import oracle
from conftest import load_golden


def test_rank_unrank_roundtrip():
    import ctypes
    lib = oracle.load()
    lib.orc_rank.restype = ctypes.c_uint64
    lib.orc_rank.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    lib.orc_unrank.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p]
    rng = np.random.default_rng(1)
    for n, k in ((16, 5), (25, 6)):
        total = int(np.prod([n - i for i in range(k)]))
        for r in list(rng.integers(0, total, 200)) + [0, total - 1]:
            pos = np.zeros(8, dtype=np.int32)
            lib.orc_unrank(n, k, int(r), pos.ctypes.data)
            assert len(set(pos[:k].tolist())) == k and pos[:k].max() < n
            assert lib.orc_rank(n, k, pos.ctypes.data) == r


def test_pattern_partitions_cover_tiles():
    import ctypes
    lib = oracle.load()
    for w in (4, 5):
        n = w * w
        for part in (0, 1):
            seen = []
            for p in range(lib.orc_num_patterns(w)):
                tiles = np.zeros(8, dtype=np.int32)
                sym = np.zeros(25, dtype=np.int32)
                assert lib.orc_pattern(w, part, p, tiles.ctypes.data, sym.ctypes.data) >= 0
                seen += tiles[: lib.orc_pattern_k(w)].tolist()
            assert sorted(seen) == list(range(1, n)), (w, part)


def test_manhattan_all_solutions_golden():
    """benchmarks/manhattan_expand_nodes.csv rows 0-12 (the fast ones)."""
    g = load_golden("yama24_hard_new.json")["instances"][:13]
    res = oracle.solve(5, [x["tiles"] for x in g], oracle.MD)
    for x, r in zip(g, res):
        assert (r["len"], r["nodes_total"]) == tuple(x["md"]), x["name"]
        assert r["nodes_total"] == sum(r["nodes"])
        assert r["f_limit"][-1] >= r["len"]


def test_pdb_all_solutions_golden(pdb24_tables):
    """All 50 rows of benchmarks/pdb_expand_nodes.csv: pins the PDB semantics."""
    g = load_golden("yama24_hard_new.json")["instances"]
    res = oracle.solve(5, [x["tiles"] for x in g], oracle.PDB, pdb24_tables)
    for x, r in zip(g, res):
        assert (r["len"], r["nodes_total"]) == tuple(x["pdb"]), x["name"]


def test_pdb_first_solution_golden(pdb24_tables):
    """test/result_24puzzle.txt lines 53-102 (first-solution PDB solver).  Line 52
    (prob000) repeats the Manhattan block's value 50196 and is excluded."""
    g = load_golden("yama24_med.json")["instances"]
    res = oracle.solve(5, [x["tiles"] for x in g], oracle.PDB, pdb24_tables, mode=oracle.FIRST)
    for x, r in zip(g, res):
        if x["name"] == "prob000":
            assert x["pdb_first"] == x["md_first"]
            continue
        assert (r["len"], r["nodes_total"]) == tuple(x["pdb_first"]), x["name"]


def test_manhattan_first_solution_golden():
    """test/result_24puzzle.txt lines 103-153, compared modulo 2^32: the
    reference's `int node_num` wraps (prob018: 8611234222 mod 2^32 = 21299630).
    Rows above 2e7 nodes are skipped to keep the CPU suite short."""
    g = [x for x in load_golden("yama24_med.json")["instances"] if x["md_first"][1] < 20_000_000]
    res = oracle.solve(5, [x["tiles"] for x in g], oracle.MD, mode=oracle.FIRST)
    for x, r in zip(g, res):
        assert r["len"] == x["md_first"][0], x["name"]
        assert r["nodes_total"] % (1 << 32) == x["md_first"][1], x["name"]


def test_korf100_lengths_pdb555(pdb15_tables):
    """Optimal lengths of test/result_15puzzle.txt with the 5-5-5 PDB (the
    reference has no 15-puzzle PDB; equal optimal lengths pin admissibility)."""
    g = load_golden("korf100.json")["instances"][:40]
    res = oracle.solve(4, [x["tiles"] for x in g], oracle.PDB, pdb15_tables)
    for x, r in zip(g, res):
        assert r["len"] == x["len"], x["name"]


def test_korf100_md_equals_pdb_lengths(pdb15_tables):
    g = load_golden("korf100.json")["instances"]
    easy = [g[i]["tiles"] for i in (1, 2, 4, 7, 21)]
    a = oracle.solve(4, easy, oracle.MD)
    b = oracle.solve(4, easy, oracle.PDB, pdb15_tables)
    assert [r["len"] for r in a] == [r["len"] for r in b]


def test_pdb_fingerprints(pdb15_tables, pdb24_tables):
    fp = load_golden("pdb_fingerprints.json")["tables"]
    for w, tabs in ((4, pdb15_tables), (5, pdb24_tables)):
        for t, arr in enumerate(tabs):
            assert hashlib.sha256(arr.tobytes()).hexdigest() == fp["%d_%d" % (w, t)]["sha256"]


def test_pdb_admissible_dominates_pattern_md(pdb15_tables):
    """h_PDB >= Manhattan distance of the pattern tiles, on random states."""
    import instances
    states = instances.random_permutations(4, 200, seed=7)
    hp = oracle.heuristic(4, states, oracle.PDB, pdb15_tables)
    hm = oracle.heuristic(4, states, oracle.MD)
    assert np.all(hp >= hm)


def test_edge_cases():
    goal = list(range(16))
    r = oracle.solve(4, [goal], oracle.MD)[0]
    # the goal is expanded once: its 2 children are generated and pruned
    assert (r["status"], r["len"], r["nodes_total"], r["n_iter"]) == (0, 0, 2, 1)
    bad = list(range(16))
    bad[3] = 2
    assert oracle.solve(4, [bad], oracle.MD)[0]["status"] == -2
    unsolvable = list(range(16))
    unsolvable[1], unsolvable[2] = unsolvable[2], unsolvable[1]
    assert oracle.solve(4, [unsolvable], oracle.MD)[0]["status"] == -3
    one = list(range(16))
    one[0], one[1] = 1, 0
    r = oracle.solve(4, [one], oracle.MD)[0]
    assert r["len"] == 1 and r["moves"] == bytes([2])
    assert oracle.solve(4, np.zeros((0, 16), np.uint8), oracle.MD) == []


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(oracle.__file__), "_ref", "bin", "24puzzle_expand")),
                    reason="reference CPU solvers not compiled here (oracle/_ref)")
def test_oracle_matches_reference_binaries(pdb24_tables):
    import ref_run
    import instances
    states = instances.random_walks(5, 10, 46, seed=99)
    got = oracle.solve(5, states, oracle.MD)
    ref = ref_run.run_md24_expand(states)
    assert [(r["len"], r["nodes_total"] % (1 << 32)) for r in got] == [(a, b % (1 << 32)) for a, b in ref]
    gotp = oracle.solve(5, states, oracle.PDB, pdb24_tables)
    refp = ref_run.run_pdb24_expand(states, pdb24_tables)
    assert [(r["len"], r["nodes_total"]) for r in gotp] == refp


def test_split_driver_matches_serial_search(pdb15_tables):
    """orc_solve_batch_split (every host thread on one instance, the CPU
    baseline's driver) gives the serial search's lengths and per-iteration
    counts, and valid paths, for both heuristics and both widths."""
    import instances
    import slide
    cases = [(4, oracle.MD, instances.random_walks(4, 24, (40, 70), seed=3), None),
             (4, oracle.PDB, instances.random_permutations(4, 6, seed=5), pdb15_tables),
             (5, oracle.MD, instances.random_walks(5, 6, 40, seed=6), None),
             (4, oracle.MD, np.arange(16, dtype=np.uint8)[None, :], None)]
    for w, heur, states, tabs in cases:
        a = oracle.solve(w, states, heur, tabs)
        for threads in (1, 3, 8):
            b = oracle.solve(w, states, heur, tabs, threads=threads, split=True)
            for i, (x, y) in enumerate(zip(a, b)):
                assert (y["status"], y["len"], y["f_limit"], y["nodes"]) == \
                    (x["status"], x["len"], x["f_limit"], x["nodes"]), (w, heur, threads, i)
                assert slide.is_solution(states[i], y["moves"], w), (w, heur, threads, i)


def test_first_path_restatement_semantics():
    """orc_first_path, the CPU statement of Horie's per-root search: a root
    finds a goal exactly when f_limit reaches its optimal length (Manhattan
    is admissible), the path replays to the goal within f_limit, and it is
    the first in depth-first order -- here checked as: never shorter than
    optimal, and equal to optimal when f_limit is the optimal length."""
    import instances
    import slide
    states = instances.random_walks(4, 24, (8, 30), seed=3)
    opt = [r["len"] for r in oracle.solve(4, states, oracle.MD)]
    for f in (0, 9, 14, 20, 26):
        rows = oracle.first_paths(states, f)
        for i, r in enumerate(rows):
            L = int(r[0])
            if f < opt[i]:
                assert L == -1, (f, i)
                continue
            assert opt[i] <= L <= f and (L - opt[i]) % 2 == 0, (f, i)
            assert slide.is_solution(states[i], bytes(r[1:1 + L].astype(np.uint8)), 4), (f, i)
    exact = oracle.first_paths(states[:1], opt[0])
    assert int(exact[0][0]) == opt[0]
    goal = oracle.first_paths(np.arange(16, dtype=np.uint8), 0)
    assert int(goal[0][0]) == 0
