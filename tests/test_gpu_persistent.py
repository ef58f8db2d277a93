"""GPU parity of the multi-iteration (persistent) mode: every instance runs
its own threshold loop on the device inside one launch (handback_nodes = 0),
and of the hybrid that hands large iterations back to the round loop.  Same
answers, bit for bit, as the oracle and the reference's golden rows."""
import numpy as np
import pytest

import instances
import oracle
import slide
from conftest import load_golden
from test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("lb", ["steal", "static", "none"])
def test_persistent_md15_walks(gpu_solver, lb):
    w, states = instances.config_instances("15_md_walk60")
    s = gpu_solver(w, "manhattan")
    s.set_config(persistent=1, handback_nodes=0, lb_mode=lb, frontier_target=256 if lb != "none" else 2048)
    want = oracle.solve(w, states, oracle.MD)
    got = s.solve(states)
    for i, (a, b) in enumerate(zip(got, want)):
        assert_same(a, b, states[i], w, "%s/walk%d" % (lb, i))
    st = s.stats()
    assert st["kernel_launches"] <= 3  # pool set-up + one search launch (+ heuristic)


def test_persistent_mixed_depths(gpu_solver):
    """Instances finishing many iterations apart share the one launch."""
    s = gpu_solver(4, "manhattan")
    states = np.concatenate([instances.random_walks(4, 20, (5, 30), seed=31),
                             instances.random_walks(4, 20, (60, 100), seed=32)])
    s.set_config(persistent=1, handback_nodes=0, frontier_target=64)
    want = oracle.solve(4, states, oracle.MD)
    got = s.solve(states)
    for i, (a, b) in enumerate(zip(got, want)):
        assert_same(a, b, states[i], 4, "mixed%d" % i)


def test_persistent_pdb24_golden_rows(gpu_solver, pdb24_tables):
    g = load_golden("yama24_hard_new.json")["instances"]
    states = np.array([x["tiles"] for x in g], dtype=np.uint8)
    s = gpu_solver(5, "pdb")
    s.set_config(persistent=1, handback_nodes=0)
    got = s.solve(states)
    for x, a, t in zip(g, got, states):
        assert a["status"] == 0, x["name"]
        assert (a["len"], a["nodes_total"]) == tuple(x["pdb"]), x["name"]
        assert slide.is_solution(t, a["moves"], 5), x["name"]
    want = oracle.solve(5, states[:8], oracle.PDB, pdb24_tables)
    for i in range(8):
        assert_same(got[i], want[i], states[i], 5, g[i]["name"])


def test_persistent_md24_golden(gpu_solver):
    g = load_golden("yama24_hard_new.json")["instances"][:13]
    states = np.array([x["tiles"] for x in g], dtype=np.uint8)
    s = gpu_solver(5, "manhattan")
    s.set_config(persistent=1, handback_nodes=0, lb_mode="static")
    got = s.solve(states)
    want = oracle.solve(5, states, oracle.MD)
    for x, a, b, t in zip(g, got, want, states):
        assert (a["len"], a["nodes_total"]) == tuple(x["md"]), x["name"]
        assert_same(a, b, t, 5, x["name"])


def test_persistent_pdb15_random(gpu_solver, pdb15_tables):
    states = instances.random_permutations(4, 12, seed=0x15B)
    s = gpu_solver(4, "pdb")
    s.set_config(persistent=1, handback_nodes=0, lb_mode="static")
    got = s.solve(states)
    want = oracle.solve(4, states, oracle.PDB, pdb15_tables)
    for i, (a, b) in enumerate(zip(got, want)):
        assert_same(a, b, states[i], 4, "rand%d" % i)


def test_persistent_donation_under_pressure(gpu_solver):
    s = gpu_solver(5, "manhattan")
    g = load_golden("yama24_hard_new.json")["instances"][10:12]
    states = np.array([x["tiles"] for x in g], dtype=np.uint8)
    s.set_config(persistent=1, handback_nodes=0, frontier_target=4, donate_min_slack=4)
    got = s.solve(states)
    for x, a, t in zip(g, got, states):
        assert (a["len"], a["nodes_total"]) == tuple(x["md"]), x["name"]
        assert slide.is_solution(t, a["moves"], 5)
    assert s.stats()["tasks_donated"] > 1000


def test_persistent_edge_cases(gpu_solver):
    s = gpu_solver(4, "manhattan")
    s.set_config(persistent=1, handback_nodes=0)
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
    assert res[2]["status"] == -2 and res[3]["status"] == -3
    assert s.solve(np.zeros((0, 16), np.uint8)) == []


def test_persistent_matches_round_mode(gpu_solver):
    s = gpu_solver(4, "pdb")
    states = instances.random_permutations(4, 6, seed=77)
    s.set_config(persistent=0)
    a = [(r["len"], r["nodes"], r["f_limit"]) for r in s.solve(states)]
    s.set_config(persistent=1, handback_nodes=0)
    b = [(r["len"], r["nodes"], r["f_limit"]) for r in s.solve(states)]
    assert a == b


@pytest.mark.parametrize("handback", [1, 2000, 200000])
def test_hybrid_handback_keeps_counts(gpu_solver, handback):
    """Persistent loop first, then the round loop for instances whose
    iterations grew past `handback` nodes: the same answers."""
    w, states = instances.config_instances("15_md_walk60")
    s = gpu_solver(w, "manhattan")
    s.set_config(persistent=1, handback_nodes=handback, frontier_target=256)
    want = oracle.solve(w, states, oracle.MD)
    got = s.solve(states)
    for i, (a, b) in enumerate(zip(got, want)):
        assert_same(a, b, states[i], w, "hb%d/%d" % (handback, i))


def test_hybrid_pdb24_golden(gpu_solver):
    g = load_golden("yama24_hard_new.json")["instances"][:10]
    states = np.array([x["tiles"] for x in g], dtype=np.uint8)
    s = gpu_solver(5, "pdb")
    s.set_config(persistent=1, handback_nodes=1000000)
    got = s.solve(states)
    for x, a, t in zip(g, got, states):
        assert a["status"] == 0, x["name"]
        assert (a["len"], a["nodes_total"]) == tuple(x["pdb"]), x["name"]
        assert slide.is_solution(t, a["moves"], 5), x["name"]
