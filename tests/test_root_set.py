"""Root-set templates (host logic, no GPU): the uniform-depth tree the batch
solve expands below every instance (the counterpart of create_root_set,
src/24puzzle_block_parallel_with_pdb.cu:454-490), checked against an
independent breadth-first expansion written here."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "sliding-puzzle_gb300"))
import slide  # noqa: E402


def _bfs(width, blank, target):
    """Level-by-level expansion, children in move order (0 up, 1 right,
    2 left, 3 down), no move reversing its parent's; stops at the first
    level with at least `target` nodes.  Returns (paths, depth, leaves)."""
    delta = (-width, 1, -1, width)

    def legal(cell):
        r, c = divmod(cell, width)
        return [r > 0, c < width - 1, c > 0, r < width - 1]

    nodes = [(0, blank, -1, 0)]  # (path, cell, incoming move, depth)
    level = [0]
    depth = 0
    while len(level) < target:
        nxt = []
        for x in level:
            path, cell, pre, dep = nodes[x]
            ok = legal(cell)
            for d in range(4):
                if not ok[d] or (pre >= 0 and d == 3 - pre):
                    continue
                nodes.append((path | (d << (2 * dep)), cell + delta[d], d, dep + 1))
                nxt.append(len(nodes) - 1)
        level = nxt
        depth += 1
    return [p for p, _, _, _ in nodes], depth, len(level)


@pytest.mark.parametrize("width", [4, 5])
@pytest.mark.parametrize("target", [1, 2, 37, 512, 2048])
def test_template_matches_breadth_first_expansion(width, target):
    for blank in range(width * width):
        paths, depth, leaves = _bfs(width, blank, target)
        n, d, nl, got = slide.root_set_template(width, blank, target, cap=len(paths))
        assert (n, d, nl) == (len(paths), depth, leaves), (width, blank, target)
        assert np.array_equal(got, np.array(paths, dtype=np.uint64)), (width, blank, target)
        assert nl >= target


def test_template_replays_to_distinct_paths_of_its_depth():
    # every leaf is a legal non-backtracking walk of exactly D moves
    n, d, nl, paths = slide.root_set_template(4, 5, 3072, cap=1 << 16)
    leaves = paths[n - nl:]
    assert len(set(int(p) for p in leaves)) == nl
    for p in leaves[:: max(1, nl // 200)]:
        cell, pre = 5, -1
        for j in range(d):
            mv = (int(p) >> (2 * j)) & 3
            assert pre < 0 or mv != 3 - pre
            r, c = divmod(cell, 4)
            assert [r > 0, c < 3, c > 0, r < 3][mv]
            cell += (-4, 1, -1, 4)[mv]
            pre = mv


def test_template_argument_checks():
    lib = slide.load()
    import ctypes
    n, d, nl = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
    for args in ((3, 0, 8), (4, 16, 8), (4, -1, 8), (4, 0, 0), (5, 25, 8), (4, 0, (1 << 20) + 1)):
        st = lib.sp_root_set_template(args[0], args[1], args[2], None, 0, ctypes.byref(n), ctypes.byref(d),
                                      ctypes.byref(nl))
        assert st == -1, args


def test_template_at_the_largest_target():
    # the largest configurable root set (2^20 per instance) stays within the
    # 64-bit move encoding and the 24-bit node numbering of the goal records
    for width, blank in ((4, 0), (5, 12)):
        n, d, nl, _ = slide.root_set_template(width, blank, 1 << 20)
        assert nl >= 1 << 20 and d <= 32 and n < 1 << 24
