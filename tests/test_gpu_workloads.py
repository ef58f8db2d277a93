"""GPU parity on the benchmark workloads themselves, in the library's default
mode (hybrid threshold loop: small iterations in one persistent launch,
iterations predicted at 600000 nodes or more handed to the host round
loop), and the reference-format table import.

Every instance of the headline workload is compared with the oracle:
per-iteration f-limits and node counts, the optimal length and a replayed
path.  Integer work, so every comparison is exact."""
import numpy as np
import pytest

import bench
import instances
import oracle
import slide
from conftest import load_golden
from test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def headline():
    w, states = bench.workload(0)
    want = oracle.solve(w, states, oracle.PDB, oracle.tables(w))
    return w, states, want


def test_headline_workload_all_instances_default_mode(gpu_solver, headline):
    """All 100 instances of the benchmark's 15-puzzle 5-5-5 PDB workload,
    through sp_solve_batch with the default configuration."""
    w, states, want = headline
    s = gpu_solver(w, "pdb")
    cfg = slide.default_config()
    assert s.config.persistent == 1 and s.config.handback_nodes == cfg.handback_nodes == 600000
    got = s.solve(states)
    for i, (a, b) in enumerate(zip(got, want)):
        assert_same(a, b, states[i], w, "headline%d" % i)
    st = s.stats()
    assert st["nodes"] == sum(x["nodes_total"] for x in want)
    # the hybrid loop really ran both phases on this workload
    assert st["rounds"] >= 1 and st["tasks_donated"] > 0


def test_headline_workload_device_entry_point(gpu_solver, headline):
    """The call the benchmark times (instances already in device memory),
    twice in a row, against the oracle."""
    import torch
    w, states, want = headline
    s = gpu_solver(w, "pdb")
    d = torch.from_numpy(states.copy()).cuda()
    for rep in range(2):
        res = s.solve_device_raw(d.data_ptr(), states.shape[0])
        for i in range(states.shape[0]):
            assert_same(slide.result_dict(res[i]), want[i], states[i], w, "device%d/%d" % (rep, i))


@pytest.mark.parametrize("width", [4, 5])
def test_pdb_import_reference_order_round_trip(width, pdb15_tables, pdb24_tables):
    """Tables in the reference's table-file byte order (the oracle's compact
    rank order), imported into a solver that never built its own: usable
    only once every table is in, exported back byte for byte, and solving
    the golden rows with the reference's counts."""
    tabs = pdb15_tables if width == 4 else pdb24_tables
    with slide.Solver(width, "pdb") as s:
        probe = instances.random_permutations(width, 4, seed=8)
        with pytest.raises(slide.SlideError) as e:
            s.heuristic_values(probe)
        assert e.value.status == -6  # SP_ERR_NO_PDB
        with pytest.raises(slide.SlideError) as e:
            s.import_pdb(0, tabs[0][:-1])
        assert e.value.status == -1
        for t, arr in enumerate(tabs):
            if t + 1 < len(tabs):
                s.import_pdb(t, arr)
                with pytest.raises(slide.SlideError):
                    s.heuristic_values(probe)
            else:
                s.import_pdb(t, arr)
        for t, arr in enumerate(tabs):
            assert np.array_equal(s.export_pdb(t), arr), t
        assert np.array_equal(s.heuristic_values(probe), oracle.heuristic(width, probe, oracle.PDB, tabs))
        if width == 5:
            g = load_golden("yama24_hard_new.json")["instances"][:10]
            states = np.array([x["tiles"] for x in g], dtype=np.uint8)
            got = s.solve(states)
            for x, a, t in zip(g, got, states):
                assert a["status"] == 0, x["name"]
                assert (a["len"], a["nodes_total"]) == tuple(x["pdb"]), x["name"]
                assert slide.is_solution(t, a["moves"], 5), x["name"]
        else:
            g = load_golden("korf100.json")["instances"][:10]
            states = np.array([x["tiles"] for x in g], dtype=np.uint8)
            got = s.solve(states)
            want = oracle.solve(4, states, oracle.PDB, tabs)
            for x, a, b, t in zip(g, got, want, states):
                assert a["len"] == x["len"], x["name"]
                assert_same(a, b, t, 4, x["name"])


# Instances of each 24-puzzle bin (50 seeded walks of 120 / 160 / 200 moves)
# that the oracle solves with fewer than 15 M generated nodes: found once by
# running the oracle over every instance of the bins with a node budget.
# The harder instances of the bins cost the oracle minutes to hours each.
BIN_ORACLE_SAMPLE = {
    120: [7, 22, 5, 8, 23, 42, 30, 46, 25, 3, 40, 33, 2, 41, 14, 32, 24, 29, 35, 49, 44, 10, 19, 13, 28, 38,
          6, 37, 4, 48],
    160: [10, 8, 38, 18, 13, 14, 2, 47, 9, 22, 12, 17, 40, 35, 41, 21, 26],
    200: [48, 31, 22, 35, 37, 1, 6, 16, 23, 45, 26],
}


@pytest.mark.parametrize("walk", [120, 160, 200])
def test_24_bins_default_mode_against_oracle(gpu_solver, pdb24_tables, walk):
    """A bin of the 24-puzzle workload solved as the benchmark solves it
    (whole bin in one batch, 8192 roots per instance, default threshold
    loop); every answer is a replayed optimal-length path, and the sampled
    instances match the oracle iteration by iteration."""
    w, states = instances.config_instances("24_walk%d" % walk)
    s = gpu_solver(5, "pdb")
    s.set_config(frontier_target=8192)
    got = s.solve(states)
    h0 = oracle.heuristic(5, states, oracle.PDB, pdb24_tables)
    for i, a in enumerate(got):
        assert a["status"] == 0, i
        assert a["len"] >= h0[i] and (a["len"] - h0[i]) % 2 == 0, i
        assert slide.is_solution(states[i], a["moves"], 5), i
    idx = BIN_ORACLE_SAMPLE[walk]
    want = oracle.solve(5, states[idx], oracle.PDB, pdb24_tables)
    for j, i in enumerate(idx):
        assert_same(got[i], want[j], states[i], 5, "24_walk%d/%d" % (walk, i))
