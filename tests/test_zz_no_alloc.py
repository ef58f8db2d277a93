"""sp_dfs_round_md_noalloc: the threshold round that allocates no memory.

It serves callers that cannot call cudaMalloc -- hosts whose framework owns
the device allocator and must account for every byte, real-time loops that
must not enter the driver's allocator.  The caller passes device buffers for
inputs and outputs; the round's scratch lives in a fixed device array inside
the library.  These tests call it through the C ABI and compare it with
sp_dfs_round (which allocates through its solver handle) and with a plain
Python count: node counts are integers, so they must be equal, on two calls
in a row and across widths.  This file runs last so a failure here leaves
every other test already run.
"""
import ctypes

import numpy as np
import pytest

import instances
import slide

pytestmark = pytest.mark.gpu

SP_ERR_CAPACITY = -9


@pytest.fixture(scope="module")
def lib():
    l = slide.load()
    f = l.sp_dfs_round_md_noalloc
    f.restype = ctypes.c_int32
    f.argtypes = [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                  ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return l


def noalloc_round(lib, width, roots, depth, pre, limit):
    import torch
    n = len(roots)
    d_roots = torch.from_numpy(np.ascontiguousarray(roots, dtype=np.uint8)).cuda()
    d_depth = torch.tensor(np.asarray(depth, dtype=np.int32)).cuda()
    d_pre = torch.tensor(np.asarray(pre, dtype=np.int32)).cuda()
    # stale values: the call must overwrite every output
    d_nodes = torch.full((max(n, 1),), 987654321, dtype=torch.int64, device="cuda")
    d_found = torch.full((1,), 777, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = lib.sp_dfs_round_md_noalloc(width, d_roots.data_ptr(), d_depth.data_ptr(), d_pre.data_ptr(), n,
                                     int(limit), d_nodes.data_ptr(), d_found.data_ptr(), None)
    torch.cuda.synchronize()
    return st, d_nodes[:n].cpu().numpy().astype(np.uint64), int(d_found.item())


def round_set(width, n, seed, walk):
    roots = instances.random_walks(width, n, walk, seed=seed)
    depth = (np.arange(n) % 4).astype(np.int32)
    pre = (np.arange(n) % 5 - 1).astype(np.int32)  # -1 .. 3
    return roots, depth, pre


def test_two_calls_match_allocating_round(lib):
    with slide.Solver(4, "manhattan") as s:
        for call, (seed, walk, slack) in enumerate(((11, 30, 10), (12, 40, 12))):
            roots, depth, pre = round_set(4, 3000, seed, walk)
            limit = int(np.median(s.heuristic_values(roots))) + slack
            want_nodes, want_found = s.dfs_round(roots, depth, pre, limit)
            st, nodes, found = noalloc_round(lib, 4, roots, depth, pre, limit)
            assert st == 0, (call, st)
            assert np.array_equal(nodes, want_nodes), call
            assert found == want_found, call
            assert nodes.sum() > 0


def test_width5_and_goal_root(lib):
    with slide.Solver(5, "manhattan") as s:
        roots, depth, pre = round_set(5, 500, 21, 36)
        roots[7] = np.arange(25, dtype=np.uint8)  # a goal root: found = its depth or less
        limit = int(np.median(s.heuristic_values(roots))) + 6
        for _ in range(2):
            want_nodes, want_found = s.dfs_round(roots, depth, pre, limit)
            st, nodes, found = noalloc_round(lib, 5, roots, depth, pre, limit)
            assert st == 0
            assert np.array_equal(nodes, want_nodes)
            assert found == want_found and 0 <= found <= depth[7]


def test_rejects_oversized_input_then_works(lib):
    roots, depth, pre = round_set(4, 16385, 3, 10)
    st, _, _ = noalloc_round(lib, 4, roots, depth, pre, 40)
    assert st == SP_ERR_CAPACITY
    roots, depth, pre = round_set(4, 64, 4, 20)
    with slide.Solver(4, "manhattan") as s:
        want_nodes, want_found = s.dfs_round(roots, depth, pre, 30)
    st, nodes, found = noalloc_round(lib, 4, roots, depth, pre, 30)
    assert st == 0 and np.array_equal(nodes, want_nodes) and found == want_found


def test_counts_match_pure_python_subtree_counter(lib):
    """Independent of the allocating path: every root's count and the
    shortest goal depth against a plain depth-first count in Python."""
    from test_gpu_parity import _py_subtree
    for width, walk, limit in ((4, 14, 16), (5, 12, 14)):
        roots = instances.random_walks(width, 24, walk, seed=12 + width)
        depth = (np.arange(24) % 5).astype(np.int32)
        pre = np.array([-1, 0, 1, 2, 3, -1] * 4, dtype=np.int32)
        for _ in range(2):
            st, nodes, found = noalloc_round(lib, width, roots, depth, pre, limit)
            assert st == 0
            want_found = -1
            for i in range(len(roots)):
                c, f = _py_subtree(roots[i].tolist(), width, int(depth[i]), int(pre[i]), limit)
                assert int(nodes[i]) == c, (width, i)
                if f >= 0 and (want_found < 0 or f < want_found):
                    want_found = f
            assert found == want_found, width


SP_ERR_ARG = -1
SP_ERR_NOT_PERMUTATION = -2


def test_invalid_roots_are_reported_then_a_valid_call_works(lib):
    roots, depth, pre = round_set(4, 200, 5, 20)
    bad = roots.copy()
    bad[17, 3] = bad[17, 4]  # a repeated tile
    st, _, _ = noalloc_round(lib, 4, bad, depth, pre, 40)
    assert st == SP_ERR_NOT_PERMUTATION
    bad = roots.copy()
    bad[3, 0] = 16  # not a tile of the 15-puzzle
    st, _, _ = noalloc_round(lib, 4, bad, depth, pre, 40)
    assert st == SP_ERR_NOT_PERMUTATION
    d = depth.copy()
    d[5] = -1
    st, _, _ = noalloc_round(lib, 4, roots, d, pre, 40)
    assert st == SP_ERR_ARG
    p = pre.copy()
    p[9] = 4
    st, _, _ = noalloc_round(lib, 4, roots, depth, p, 40)
    assert st == SP_ERR_ARG
    with slide.Solver(4, "manhattan") as s:
        limit = int(np.median(s.heuristic_values(roots))) + 8
        want_nodes, want_found = s.dfs_round(roots, depth, pre, limit)
    st, nodes, found = noalloc_round(lib, 4, roots, depth, pre, limit)
    assert st == 0 and np.array_equal(nodes, want_nodes) and found == want_found
