"""The learned balancer's training-data walks, on the CPU: valid, solvable,
seeded permutations whose blank moves never reverse (the same rule as the
search), at the distance the length range allows."""
import numpy as np

import instances
import train_lb


def test_vector_walks_are_solvable_seeded_permutations():
    for width, lo, hi in ((4, 40, 80), (5, 100, 220)):
        a = train_lb.vector_walks(width, 300, lo, hi, seed=11)
        b = train_lb.vector_walks(width, 300, lo, hi, seed=11)
        c = train_lb.vector_walks(width, 300, lo, hi, seed=12)
        assert a.shape == (300, width * width) and a.dtype == np.uint8
        assert np.array_equal(a, b) and not np.array_equal(a, c)
        goal = np.arange(width * width)
        for row in a:
            assert np.array_equal(np.sort(row), goal)
            assert instances.is_solvable(row, width)


def test_vector_walk_length_bounds_manhattan_distance():
    # each of the m moves slides one tile by one cell: the Manhattan distance
    # changes by +-1 per move, so it is at most m and has m's parity
    a = train_lb.vector_walks(4, 200, 7, 7, seed=3)
    for row in a:
        md = instances.manhattan(row, 4)
        assert md <= 7 and md % 2 == 1
        blank = int(np.flatnonzero(row == 0)[0])
        # the blank's parity of (row + col) flips every move
        assert (blank // 4 + blank % 4) % 2 == 1
