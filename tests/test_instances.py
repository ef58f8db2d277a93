"""Seeded instance generators (no GPU)."""
import numpy as np

import instances
import slide


def test_xoshiro_deterministic_and_uniformish():
    a = instances.Xoshiro256ss(42)
    b = instances.Xoshiro256ss(42)
    xs = [a.next() for _ in range(100)]
    assert xs == [b.next() for _ in range(100)]
    c = instances.Xoshiro256ss(1)
    counts = np.bincount([c.below(4) for _ in range(4000)], minlength=4)
    assert counts.min() > 850


def test_random_walks_are_reachable_and_deterministic():
    for w, m in ((4, 60), (5, 120)):
        a = instances.random_walks(w, 20, m, seed=5)
        assert np.array_equal(a, instances.random_walks(w, 20, m, seed=5))
        for s in a:
            assert sorted(s.tolist()) == list(range(w * w))
            assert instances.is_solvable(s, w)
    r = instances.random_walks(4, 50, (40, 80), seed=3)
    assert r.shape == (50, 16)


def test_random_permutations_solvable_and_varied():
    for w in (4, 5):
        a = instances.random_permutations(w, 200, seed=11)
        assert all(instances.is_solvable(s, w) for s in a)
        assert len({s.tobytes() for s in a}) == 200
        # blank lands anywhere
        assert len(set(int(np.flatnonzero(s == 0)[0]) for s in a)) > w * w // 2


def test_reference_walks_reach_md_threshold():
    a = instances.reference_walks(5, 6, seed=1, md_min=30)
    assert all(instances.manhattan(s, 5) >= 30 for s in a)


def test_replay_helper():
    s = instances.random_walks(4, 1, 10, seed=2)[0]
    assert not slide.is_solution(s, b"", 4) or np.array_equal(s, np.arange(16))
    g = np.arange(16, dtype=np.uint8)
    assert slide.is_solution(g, b"", 4)
    one = g.copy()
    one[0], one[1] = 1, 0
    assert slide.is_solution(one, bytes([2]), 4)


def test_benchmark_configurations():
    """The seeded workloads of the benchmark plan: sizes, widths, solvable
    permutations, reproducible, and the bench headline's batch is the
    `15_random` configuration."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    want = {"15_md_walk60": (4, 100), "15_random": (4, 100), "15_mixed4096": (4, 4096),
            "24_walk120": (5, 50), "24_walk160": (5, 50), "24_walk200": (5, 50)}
    for name, (w, n) in want.items():
        gw, a = instances.config_instances(name)
        assert (gw, a.shape, a.dtype) == (w, (n, w * w), np.uint8), name
        gw2, b = instances.config_instances(name)
        assert np.array_equal(a, b), name
        assert all(instances.is_solvable(s, w) for s in a), name
        assert all(sorted(s.tolist()) == list(range(w * w)) for s in a), name
    # walks stay within their length in Manhattan distance
    _, md60 = instances.config_instances("15_md_walk60")
    assert max(instances.manhattan(s, 4) for s in md60) <= 60
    _, mixed = instances.config_instances("15_mixed4096")
    assert max(instances.manhattan(s, 4) for s in mixed[:2048]) <= 80
    w, head = bench.workload(0)
    assert w == 4 and np.array_equal(head, instances.config_instances("15_random")[1])
    try:
        instances.config_instances("nope")
    except KeyError:
        pass
    else:
        raise AssertionError("unknown configuration accepted")
