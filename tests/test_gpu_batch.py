"""The largest batch configuration (4096 mixed 15-puzzle instances, PDB) on
the GPU: every instance solved with a valid path and a completion time
within the batch's, a seeded sample of them bit-identical to the oracle."""
import numpy as np
import pytest

import instances
import oracle
import slide
from test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu


def test_batch_4096_mixed(gpu_solver, pdb15_tables):
    w, states = instances.config_instances("15_mixed4096")
    s = gpu_solver(w, "pdb")
    got = s.solve(states)
    st = s.stats()
    assert len(got) == 4096
    for i, (r, t) in enumerate(zip(got, states)):
        assert r["status"] == 0, i
        assert len(r["moves"]) == r["len"] and slide.is_solution(t, r["moves"], w), i
        assert 0.0 < r["seconds"] <= st["wall_ms"] / 1000.0 + 1e-6, i
    pick = np.random.default_rng(4096).choice(4096, 32, replace=False)
    want = oracle.solve(w, states[pick], oracle.PDB, pdb15_tables)
    for i, b in zip(pick, want):
        assert_same(got[i], b, states[i], w, "batch/%d" % i)
