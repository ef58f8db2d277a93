"""sp_idas_parallel, the drop-in for the reference's one host-callable C
function (Horie's idas_parallel_main, src_horie/idas_parallel_host.h:33-34):
every root searched on its own to an f-limit, its first goal path in
depth-first order returned.  Plan rows are compared byte for byte with the
oracle's statement of the same search (orc_first_path); the order of moves,
the reverse-move rule, the f-test and the stop at the first goal all show in
which path comes back."""
import numpy as np
import pytest

import instances
import oracle
import slide

pytestmark = pytest.mark.gpu


def _reference_tables():
    """The reference's init_mdist and init_movable_table
    (src_horie/idas_parallel_host.c:88-129), in its layouts."""
    hd = np.zeros((16, 16, 4), np.int8)
    mv = np.zeros((16, 4), np.uint8)
    for t in range(16):
        gx, gy = t % 4, t // 4
        for i in range(16):
            x, y = i % 4, i // 4
            hd[t, i, 0] = -1 if gy > y else 1
            hd[t, i, 1] = -1 if gx < x else 1
            hd[t, i, 2] = -1 if gx > x else 1
            hd[t, i, 3] = -1 if gy < y else 1
    for i in range(16):
        x, y = i % 4, i // 4
        mv[i] = [y > 0, x < 3, x > 0, y < 3]
    return hd, mv


def _gpu_rows(roots, f_limit, hd=None, mv=None):
    import torch
    torch.cuda.set_device(0)
    n = roots.shape[0]
    d_in = torch.from_numpy(np.ascontiguousarray(roots, dtype=np.uint8)).cuda()
    d_plan = torch.full((max(n, 1), slide.SP_PLAN_STRIDE), 99, dtype=torch.int8, device="cuda")
    d_hd = torch.from_numpy(hd.reshape(-1).copy()).cuda() if hd is not None else None
    d_mv = torch.from_numpy(mv.reshape(-1).copy()).cuda() if mv is not None else None
    torch.cuda.synchronize()
    slide.idas_parallel(d_in.data_ptr(), n, d_plan.data_ptr(), f_limit,
                        d_hd.data_ptr() if d_hd is not None else None,
                        d_mv.data_ptr() if d_mv is not None else None)
    torch.cuda.synchronize()
    return d_plan[:n].cpu().numpy()


def _same(got, want):
    assert got.shape == want.shape
    for i in range(got.shape[0]):
        L = int(want[i, 0])
        assert int(got[i, 0]) == L, i
        if L > 0:
            assert np.array_equal(got[i, 1:1 + L], want[i, 1:1 + L]), i


def test_first_paths_match_the_oracle_over_f_limits():
    """A root set like the reference's distributor builds (states a few moves
    from each other and from the goal), searched at every f-limit from the
    smallest h upward, as the reference's host loop does."""
    roots = np.concatenate([instances.random_walks(4, 1500, (6, 40), seed=41),
                            np.arange(16, dtype=np.uint8)[None, :]])
    h = oracle.heuristic(4, roots, oracle.MD)
    assert h.min() == 0
    for f in list(range(0, 41, 5)) + [23, 36]:
        want = oracle.first_paths(roots, f)
        _same(_gpu_rows(roots, f), want)
    assert (want[:, 0] >= 0).sum() > 1000


def test_caller_tables_are_the_ones_searched():
    """The reference's own tables give the built-in answer; a movable table
    that forbids some moves changes the search, on the GPU exactly as in the
    oracle."""
    roots = instances.random_walks(4, 400, (10, 30), seed=42)
    hd, mv = _reference_tables()
    f = 24
    want = oracle.first_paths(roots, f)
    _same(_gpu_rows(roots, f, hd, mv), want)
    mv2 = mv.copy()
    mv2[5, 0] = 0  # the blank may not move up from cell 5
    mv2[10, 2] = 0  # nor left from cell 10
    want2 = oracle.first_paths(roots, f, hd, mv2)
    assert not np.array_equal(want2[:, 0], want[:, 0]) or any(
        not np.array_equal(a, b) for a, b in zip(want2, want))
    _same(_gpu_rows(roots, f, hd, mv2), want2)


def test_arguments_are_checked():
    lib = slide.load()
    assert lib.sp_idas_parallel(None, 0, None, 10, None, None, None) == 0
    assert lib.sp_idas_parallel(None, 4, None, 10, None, None, None) == -1
    assert lib.sp_idas_parallel(None, -1, None, 10, None, None, None) == -1
    roots = instances.random_walks(4, 4, 10, seed=1)
    with pytest.raises(slide.SlideError):
        _gpu_rows(roots, 252)
