"""GPU parity of the pure round mode (one launch per threshold round, the
host loop of src/24puzzle_block_parallel_with_pdb.cu:772-921): the library
default hands small iterations to the device loop, so this file pins the
other path explicitly."""
import numpy as np
import pytest

import instances
import oracle
import slide
from conftest import load_golden
from test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("lb", ["steal", "static", "none"])
def test_round_mode_md15_walks(gpu_solver, lb):
    w, states = instances.config_instances("15_md_walk60")
    s = gpu_solver(w, "manhattan")
    s.set_config(persistent=0, lb_mode=lb, frontier_target=256 if lb != "none" else 2048)
    want = oracle.solve(w, states, oracle.MD)
    for i, (a, b) in enumerate(zip(s.solve(states), want)):
        assert_same(a, b, states[i], w, "round/%s/%d" % (lb, i))


def test_round_mode_pdb24_golden_rows(gpu_solver):
    g = load_golden("yama24_hard_new.json")["instances"]
    states = np.array([x["tiles"] for x in g], dtype=np.uint8)
    s = gpu_solver(5, "pdb")
    s.set_config(persistent=0)
    got = s.solve(states)
    for x, a, t in zip(g, got, states):
        assert a["status"] == 0, x["name"]
        assert (a["len"], a["nodes_total"]) == tuple(x["pdb"]), x["name"]
        assert slide.is_solution(t, a["moves"], 5), x["name"]


def test_round_mode_pdb15_random(gpu_solver, pdb15_tables):
    states = instances.random_permutations(4, 12, seed=0x15B)
    s = gpu_solver(4, "pdb")
    s.set_config(persistent=0)
    want = oracle.solve(4, states, oracle.PDB, pdb15_tables)
    for i, (a, b) in enumerate(zip(s.solve(states), want)):
        assert_same(a, b, states[i], 4, "round/rand%d" % i)
