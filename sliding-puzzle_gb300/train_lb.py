"""Training data and training loop of the learned load balancer.

Tuples (state, slack) -> log2(1 + generated nodes of the state's subtree at
threshold f(state) + 2*slack).  States are the ends of seeded
non-backtracking blank walks (numpy-vectorised; 100-220 moves for the
24-puzzle); labels come from the GPU search itself: one sp_dfs_round per
batch, each root given the depth L - h - 2*slack so that a single threshold
L serves roots of every h and slack (the f-test only sees g + h).  The
per-root subtree counts are the data the reference's static balancer reads
(loop_set, src/24puzzle_block_parallel_with_pdb.cu:646).

    python sliding-puzzle_gb300/train_lb.py --width 5 --tuples 2000000 --out lbm24.npy
"""
import argparse
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import slide  # noqa: E402


def vector_walks(width, n, lo, hi, seed):
    """n states at the ends of non-backtracking blank walks of lo..hi moves."""
    rng = np.random.default_rng(seed)
    N = width * width
    b = np.tile(np.arange(N, dtype=np.uint8), (n, 1))
    blank = np.zeros(n, dtype=np.int64)
    pre = np.full(n, -1, dtype=np.int64)
    steps = rng.integers(lo, hi + 1, n)
    delta = np.array([-width, 1, -1, width])
    rows = np.arange(n)
    for s in range(int(steps.max())):
        live = steps > s
        r, c = blank // width, blank % width
        legal = np.stack([r > 0, c < width - 1, c > 0, r < width - 1], axis=1)
        legal[rows, np.where(pre >= 0, 3 - pre, 0)] &= pre < 0  # no reverse move
        # uniform choice among legal moves: the largest random key over the legal ones
        key = rng.random((n, 4)) * legal
        d = np.where(live, key.argmax(axis=1), -1)
        m = d >= 0
        src = blank[m] + delta[d[m]]
        idx = rows[m]
        b[idx, blank[m]] = b[idx, src]
        b[idx, src] = 0
        blank[m] = src
        pre[m] = d[m]
    return b


def label(solver, states, slack):
    """Generated nodes of each state's subtree at threshold f + 2*slack."""
    h = solver.heuristic_values(states).astype(np.int64)
    s = np.asarray(slack, dtype=np.int64)
    L = int((h + 2 * s).max())
    depth = (L - h - 2 * s).astype(np.int32)
    if depth.max() > 255:
        raise ValueError("slack and h span more than 255 levels")
    pre = np.full(len(states), -1, dtype=np.int32)
    nodes, _ = solver.dfs_round(states, depth, pre, L)
    return nodes


def make_dataset(solver, n, smax, seed, node_budget=2e11, chunk=1 << 16, log=print):
    """Up to n tuples spread evenly over slack 0..smax, except that no slack
    value may cost more than its share of the node budget (subtrees grow
    about 9x per slack step on the 24-puzzle, so large slacks get fewer)."""
    width = solver.width
    lo, hi = (100, 220) if width == 5 else (40, 80)
    probe = vector_walks(width, 2048, lo, hi, seed ^ 0x5EED)
    mean, prev = [], 1.0
    for s in range(smax + 1):
        # probe size: about 2e10 nodes at most, from the previous slack's mean
        m = int(min(2048, max(32, 2e10 / (prev * 10.0))))
        t0 = time.time()
        prev = max(1.0, float(label(solver, probe[:m], np.full(m, s)).mean()))
        mean.append(prev)
        log("probe slack %d: %.3g nodes/root over %d roots (%.2f s)" % (s, prev, m, time.time() - t0))
    mean = np.array(mean)
    per = n / (smax + 1.0)
    counts = np.maximum(1, np.minimum(per, node_budget / (smax + 1.0) / mean)).astype(np.int64)
    log("tuples per slack: %s (about %.3g nodes)" % (counts.tolist(), float((counts * mean).sum())))
    slack = np.repeat(np.arange(smax + 1), counts)
    rng = np.random.default_rng(seed)
    rng.shuffle(slack)
    total = len(slack)
    tiles = np.empty((total, width * width), dtype=np.uint8)
    target = np.empty(total, dtype=np.float32)
    t0 = time.time()
    t_walk = t_label = 0.0
    for off in range(0, total, chunk):
        m = min(chunk, total - off)
        ta = time.time()
        st = vector_walks(width, m, lo, hi, seed + 1 + off)
        tb = time.time()
        nodes = label(solver, st, slack[off:off + m])
        t_walk += tb - ta
        t_label += time.time() - tb
        tiles[off:off + m] = st
        target[off:off + m] = np.log2(1.0 + nodes.astype(np.float64))
    log("labelled %d tuples in %.1f s (walks %.1f s, search %.1f s)" % (total, time.time() - t0, t_walk, t_label))
    return tiles, slack.astype(np.int32), target, mean


def train(solver, tiles, slack, target, epochs=3, batch=8192, lr=1e-3, seed=0, holdout=0.05, log=print):
    """Adam on the mean squared error; returns held-out metrics."""
    n = len(target)
    rng = np.random.default_rng(seed)
    perm = rng.permutation(n)
    nh = max(128, int(n * holdout))
    hold, tr = perm[:nh], perm[nh:]
    batch = max(128, batch // 128 * 128)
    steps = 0
    t0 = time.time()
    for ep in range(epochs):
        rng.shuffle(tr)
        losses = []
        for off in range(0, len(tr) - batch + 1, batch):
            idx = tr[off:off + batch]
            losses.append(solver.lbm_train_step(tiles[idx], slack[idx], target[idx], lr))
            steps += 1
        log("epoch %d: train mse %.3f (%d steps, %.1f s)" % (ep, float(np.mean(losses)), steps, time.time() - t0))
    train_s = time.time() - t0
    y = solver.lbm_predict(tiles[hold], slack[hold])
    t = target[hold]
    mse = float(np.mean((y - t) ** 2))
    ry, rt = np.argsort(np.argsort(y)), np.argsort(np.argsort(t))
    # the slack-only baseline: mean target per slack value
    base = np.zeros_like(t)
    for s in np.unique(slack[hold]):
        m = slack[tr] == s
        base[slack[hold] == s] = target[tr][m].mean() if m.any() else t.mean()
    return {"holdout": int(nh), "mse": mse, "r2": 1.0 - mse / float(np.var(t)),
            "spearman": float(np.corrcoef(ry, rt)[0, 1]), "slack_only_mse": float(np.mean((base - t) ** 2)),
            "steps": steps, "batch": batch, "train_s": train_s}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--width", type=int, default=5)
    ap.add_argument("--tuples", type=int, default=2_000_000)
    ap.add_argument("--smax", type=int, default=7)
    ap.add_argument("--epochs", type=int, default=3)
    ap.add_argument("--seed", type=int, default=0x1B)
    ap.add_argument("--budget", type=float, default=2e11)
    ap.add_argument("--out", default="")
    a = ap.parse_args()
    s = slide.Solver(a.width, "pdb")
    s.build_pdb()
    tiles, slack, target, _ = make_dataset(s, a.tuples, a.smax, a.seed, a.budget)
    s.lbm_init(a.seed)
    print(train(s, tiles, slack, target, a.epochs))
    if a.out:
        np.save(a.out, s.lbm_export())


if __name__ == "__main__":
    main()
