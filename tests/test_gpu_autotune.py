"""The autotuner on the GPU: it keeps results identical and leaves the
solver on settings from its search space."""
import pytest

import instances
import oracle
import slide
from test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu


def test_autotune_on_gpu_keeps_results(gpu_solver):
    s = gpu_solver(4, "manhattan")
    states = instances.random_walks(4, 16, (40, 70), seed=44)
    space = (("threads_per_block", (256, 128)), ("persistent", (0, 1)))
    best, hist = slide.autotune(s, states, space=space, reps=1)
    assert best["threads_per_block"] in (128, 256) and best["persistent"] in (0, 1)
    assert len(hist) >= 3
    want = oracle.solve(4, states, oracle.MD)
    for i, (a, b) in enumerate(zip(s.solve(states), want)):
        assert_same(a, b, states[i], 4, "tuned/%d" % i)
