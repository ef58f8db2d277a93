"""GPU parity: libslide through its C ABI against the CPU oracle and the
reference's golden vectors.  Integer work, so every comparison is exact."""
import hashlib

import numpy as np
import pytest

import instances
import oracle
import slide
from conftest import load_golden

pytestmark = pytest.mark.gpu


def assert_same(got, want, tiles, width, name=""):
    assert got["status"] == 0, (name, got["status"])
    assert got["len"] == want["len"], name
    assert got["f_limit"] == want["f_limit"], name
    assert got["nodes"] == want["nodes"], name
    assert got["nodes_total"] == want["nodes_total"], name
    assert len(got["moves"]) == got["len"], name
    assert slide.is_solution(tiles, got["moves"], width), name


@pytest.fixture(scope="module")
def gpu_tables(gpu_solver):
    """GPU-built tables in compact order, checked against the oracle's fingerprints."""
    fp = load_golden("pdb_fingerprints.json")["tables"]
    out = {}
    for w in (4, 5):
        s = gpu_solver(w, "pdb")
        tabs = [s.export_pdb(t) for t in range(s.num_tables())]
        for t, arr in enumerate(tabs):
            assert hashlib.sha256(arr.tobytes()).hexdigest() == fp["%d_%d" % (w, t)]["sha256"], (w, t)
        out[w] = tabs
    return out


def test_gpu_pdb_build_matches_oracle(gpu_tables):
    # width 4 also byte-for-byte against a fresh CPU build
    for t, arr in enumerate(gpu_tables[4]):
        assert np.array_equal(arr, oracle.build_table(4, t))


def test_heuristic_values(gpu_solver, gpu_tables):
    for w in (4, 5):
        states = np.concatenate([instances.random_permutations(w, 300, seed=3),
                                 instances.random_walks(w, 100, 30, seed=4)])
        got_md = gpu_solver(w, "manhattan").heuristic_values(states)
        assert np.array_equal(got_md, oracle.heuristic(w, states, oracle.MD))
        got_pdb = gpu_solver(w, "pdb").heuristic_values(states)
        assert np.array_equal(got_pdb, oracle.heuristic(w, states, oracle.PDB, gpu_tables[w]))


def test_md15_random_walks_per_iteration(gpu_solver):
    """Workload of the 15-puzzle Manhattan configuration: 100 seeded walks of 60 moves."""
    w, states = instances.config_instances("15_md_walk60")
    want = oracle.solve(w, states, oracle.MD)
    got = gpu_solver(w, "manhattan").solve(states)
    for i, (g, o) in enumerate(zip(got, want)):
        assert_same(g, o, states[i], w, "walk%d" % i)


def test_pdb15_korf_subset_per_iteration(gpu_solver, gpu_tables):
    g = load_golden("korf100.json")["instances"][:20]
    states = np.array([x["tiles"] for x in g], dtype=np.uint8)
    want = oracle.solve(4, states, oracle.PDB, gpu_tables[4])
    got = gpu_solver(4, "pdb").solve(states)
    for x, a, b, s in zip(g, got, want, states):
        assert a["len"] == x["len"]
        assert_same(a, b, s, 4, x["name"])


def test_md24_golden_and_per_iteration(gpu_solver):
    g = load_golden("yama24_hard_new.json")["instances"][:13]
    states = np.array([x["tiles"] for x in g], dtype=np.uint8)
    got = gpu_solver(5, "manhattan").solve(states)
    want = oracle.solve(5, states, oracle.MD)
    for x, a, b, s in zip(g, got, want, states):
        assert (a["len"], a["nodes_total"]) == tuple(x["md"]), x["name"]
        assert_same(a, b, s, 5, x["name"])


def test_pdb24_golden_all_rows(gpu_solver, gpu_tables):
    """All 50 rows of benchmarks/pdb_expand_nodes.csv on the GPU."""
    g = load_golden("yama24_hard_new.json")["instances"]
    states = np.array([x["tiles"] for x in g], dtype=np.uint8)
    got = gpu_solver(5, "pdb").solve(states)
    for x, a, s in zip(g, got, states):
        assert a["status"] == 0, x["name"]
        assert (a["len"], a["nodes_total"]) == tuple(x["pdb"]), x["name"]
        assert slide.is_solution(s, a["moves"], 5), x["name"]
    want = oracle.solve(5, states[:12], oracle.PDB, gpu_tables[5])
    for i in range(12):
        assert_same(got[i], want[i], states[i], 5, g[i]["name"])


@pytest.mark.parametrize("lb", ["steal", "static", "none"])
def test_load_balance_modes_keep_counts(gpu_solver, lb):
    s = gpu_solver(4, "manhattan")
    states = instances.random_walks(4, 24, (60, 90), seed=21)
    want = oracle.solve(4, states, oracle.MD)
    s.set_config(lb_mode=lb, frontier_target=256 if lb != "none" else 2048)
    got = s.solve(states)
    for i, (a, b) in enumerate(zip(got, want)):
        assert_same(a, b, states[i], 4, "%s/%d" % (lb, i))


def test_donation_under_pressure(gpu_solver):
    """Few roots, many lanes: nearly all work arrives by in-kernel donation."""
    s = gpu_solver(5, "manhattan")
    g = load_golden("yama24_hard_new.json")["instances"][10:12]
    states = np.array([x["tiles"] for x in g], dtype=np.uint8)
    s.set_config(frontier_target=4, donate_min_slack=4)
    got = s.solve(states)
    st = s.stats()
    for x, a, t in zip(g, got, states):
        assert (a["len"], a["nodes_total"]) == tuple(x["md"]), x["name"]
        assert slide.is_solution(t, a["moves"], 5)
    assert st["tasks_donated"] > 1000


def test_frontier_sizes_agree(gpu_solver):
    s = gpu_solver(4, "pdb")
    states = instances.random_permutations(4, 8, seed=5)
    base = None
    for ft in (1, 64, 2048, 16384):
        s.set_config(frontier_target=ft)
        got = [(r["len"], r["nodes"]) for r in s.solve(states)]
        base = base or got
        assert got == base, ft


def test_repeat_is_deterministic(gpu_solver):
    s = gpu_solver(4, "manhattan")
    states = instances.random_walks(4, 50, (40, 80), seed=8)
    a = [(r["len"], r["nodes"]) for r in s.solve(states)]
    b = [(r["len"], r["nodes"]) for r in s.solve(states)]
    assert a == b


def test_edge_cases(gpu_solver):
    s = gpu_solver(4, "manhattan")
    goal = np.arange(16, dtype=np.uint8)
    one = goal.copy()
    one[0], one[1] = 1, 0
    bad = goal.copy()
    bad[3] = 2
    unsolvable = goal.copy()
    unsolvable[1], unsolvable[2] = 2, 1
    res = s.solve(np.stack([goal, one, bad, unsolvable]))
    assert (res[0]["status"], res[0]["len"], res[0]["nodes"]) == (0, 0, [2])
    assert (res[1]["status"], res[1]["len"], res[1]["moves"]) == (0, 1, bytes([2]))
    assert res[1]["nodes"] == oracle.solve(4, [one])[0]["nodes"]
    assert res[2]["status"] == -2 and res[3]["status"] == -3
    assert s.solve(np.zeros((0, 16), np.uint8)) == []
    g5 = np.arange(25, dtype=np.uint8)
    r5 = gpu_solver(5, "pdb").solve(g5[None])[0]
    assert (r5["len"], r5["nodes"]) == (0, [2])


def _py_subtree(tiles, width, g, pre, limit):
    """Generated children below one root, pure Python (small cases only)."""
    b = list(tiles)
    md = lambda bb: sum(abs(c // width - t // width) + abs(c % width - t % width) for c, t in enumerate(bb) if t)
    delta = (-width, 1, -1, width)
    count = 0
    found = -1

    def dfs(blank, g, pre, h):
        nonlocal count, found
        if h == 0 and (found < 0 or g < found):
            found = g
        if g + h > limit:
            return
        r, c = divmod(blank, width)
        for d in range(4):
            ok = (d == 0 and r > 0) or (d == 1 and c < width - 1) or (d == 2 and c > 0) or (d == 3 and r < width - 1)
            if not ok or (pre >= 0 and d == 3 - pre):
                continue
            count += 1
            src = blank + delta[d]
            b[blank], b[src] = b[src], 0
            dfs(src, g + 1, d, md(b))
            b[src], b[blank] = b[blank], 0

    dfs(b.index(0), g, pre, md(b))
    return count, found


def test_dfs_round_matches_subtree_counts(gpu_solver):
    s = gpu_solver(4, "manhattan")
    roots = instances.random_walks(4, 24, 14, seed=12)
    depth = np.arange(24) % 5
    pre = np.array([-1, 0, 1, 2, 3, -1] * 4)
    limit = 16
    nodes, found = s.dfs_round(roots, depth, pre, limit)
    want_found = -1
    for i in range(len(roots)):
        c, f = _py_subtree(roots[i].tolist(), 4, int(depth[i]), int(pre[i]), limit)
        assert int(nodes[i]) == c, i
        if f >= 0 and (want_found < 0 or f < want_found):
            want_found = f
    assert found == want_found


def test_korf100_all_lengths_pdb(gpu_solver):
    """All 100 of test/result_15puzzle.txt's optimal lengths (korf100), 5-5-5 PDB."""
    g = load_golden("korf100.json")["instances"]
    states = np.array([x["tiles"] for x in g], dtype=np.uint8)
    got = gpu_solver(4, "pdb").solve(states)
    for x, a, t in zip(g, got, states):
        assert a["status"] == 0 and a["len"] == x["len"], x["name"]
        assert slide.is_solution(t, a["moves"], 4), x["name"]


@pytest.mark.parametrize("heuristic", ["pdb", "manhattan"])
def test_yama24_50_all_lengths(gpu_solver, heuristic):
    """All of test/result_24puzzle.txt's yama24_50 optimal lengths."""
    g = load_golden("yama24_50.json")["instances"]
    states = np.array([x["tiles"] for x in g], dtype=np.uint8)
    got = gpu_solver(5, heuristic).solve(states)
    for x, a, t in zip(g, got, states):
        assert a["status"] == 0 and a["len"] == x["len"], x["name"]
        assert slide.is_solution(t, a["moves"], 5), x["name"]
