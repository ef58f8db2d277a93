"""Failure handling on the GPU without a fault: a device wait that nothing
satisfies ends after its limit with SP_ERR_TIMEOUT, and the solver (and the
CUDA context) keep working."""
import time

import pytest

import instances
import oracle
from test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("heuristic", ["manhattan", "pdb"])
def test_stalled_pool_times_out_and_solver_recovers(gpu_solver, heuristic):
    s = gpu_solver(4, heuristic)
    t0 = time.perf_counter()
    status = s.selftest_stall(200)
    dt = time.perf_counter() - t0
    assert status == -8  # SP_ERR_TIMEOUT
    assert 0.15 <= dt < 10.0
    states = instances.random_walks(4, 6, (30, 50), seed=12)
    tabs = oracle.tables(4) if heuristic == "pdb" else None
    want = oracle.solve(4, states, oracle.PDB if tabs else oracle.MD, tabs)
    for i, (a, b) in enumerate(zip(s.solve(states), want)):
        assert_same(a, b, states[i], 4, "after-stall/%d" % i)
