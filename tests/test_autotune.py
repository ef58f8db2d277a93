"""The autotuner's search on the CPU, against a fake solver whose speed
depends on its settings (no GPU needed)."""
import numpy as np
import pytest

import slide


class _Res:
    def __init__(self, ln, nodes):
        self.status, self.len, self.n_iter = 0, ln, len(nodes)
        self.nodes = list(nodes)


class FakeSolver:
    """solve_raw 'takes' a time that is lowest at tpb 128, steps 16, persistent 1."""

    width = 4
    heuristic = "manhattan"

    def __init__(self, change_results_at=None):
        self.config = slide.SpConfig()
        for f, v in dict(frontier_target=2048, threads_per_block=256, blocks_per_sm=0, lb_mode=1,
                         donate_min_slack=6, steps_per_poll=32, timeout_ms=20000, static_split_cap=10,
                         donate_reserve=0, persistent=0).items():
            setattr(self.config, f, v)
        self.now = 0.0
        self.calls = 0
        self.change_results_at = change_results_at

    def set_config(self, **kw):
        for k, v in kw.items():
            setattr(self.config, k, int(v))

    def clock(self):
        return self.now

    def solve_raw(self, a):
        c = self.config
        self.now += (1.0 + (c.threads_per_block == 256) * 0.2 + abs(c.steps_per_poll - 16) * 0.01
                     + (1 - c.persistent) * 0.3 + (c.frontier_target != 2048) * 0.05)
        self.calls += 1
        nodes = [5, 50, 500]
        if self.change_results_at is not None and c.steps_per_poll == self.change_results_at:
            nodes = [5, 50, 501]
        return [_Res(3, nodes) for _ in range(a.shape[0])]


def test_autotune_finds_the_fastest_settings():
    s = FakeSolver()
    tiles = np.tile(np.arange(16, dtype=np.uint8), (3, 1))
    best, hist = slide.autotune(s, tiles, reps=1, clock=s.clock)
    assert best["threads_per_block"] == 128
    assert best["steps_per_poll"] == 16
    assert best["persistent"] == 1
    assert best["frontier_target"] == 2048
    # the solver keeps the winner
    assert s.config.threads_per_block == 128 and s.config.persistent == 1
    # every distinct candidate timed once
    assert len(hist) == len({tuple(sorted(h.items())) for h, _ in hist})


def test_autotune_rejects_settings_that_change_results():
    s = FakeSolver(change_results_at=64)
    tiles = np.tile(np.arange(16, dtype=np.uint8), (2, 1))
    with pytest.raises(RuntimeError):
        slide.autotune(s, tiles, reps=1, clock=s.clock)


def test_autotune_cache_per_gpu_puzzle_heuristic(tmp_path):
    """A cache miss tunes and stores; a hit on the same (GPU, puzzle,
    heuristic, batch size) applies the stored settings without timing; a
    different GPU or batch size misses."""
    path = str(tmp_path / "tune.json")
    s = FakeSolver()
    s.heuristic = "pdb"
    tiles = np.tile(np.arange(16, dtype=np.uint8), (3, 1))
    best, hit = slide.autotune_cached(s, tiles, "GB300", path=path, reps=1, clock=s.clock)
    assert not hit and best["threads_per_block"] == 128
    calls = s.calls
    s2 = FakeSolver()
    s2.heuristic = "pdb"
    best2, hit2 = slide.autotune_cached(s2, tiles, "GB300", path=path, reps=1, clock=s2.clock)
    assert hit2 and s2.calls == 0 and best2 == best and s2.config.threads_per_block == 128
    _, hit3 = slide.autotune_cached(FakeSolver(), tiles, "B200", path=path, reps=1)
    assert not hit3
    s4 = FakeSolver()
    s4.heuristic = "pdb"
    _, hit4 = slide.autotune_cached(s4, np.tile(tiles, (4, 1)), "GB300", path=path, reps=1, clock=s4.clock)
    assert not hit4 and calls > 0
