"""GPU parity of the learned load balancer: the tcgen05 GEMM against FP64,
forward and gradients against the FP64 restatement (with the device's bf16
rounding points), training, and solves under SP_LB_LEARNED keeping every
count."""
import numpy as np
import pytest

import instances
import lbm_oracle as lo
import oracle
import slide
from conftest import load_golden
from test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu


def _bf16_bits(x):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def _bits_to_f64(b):
    return (b.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.mark.parametrize("m,k", [(128, 64), (256, 320), (384, 1024)])
def test_tcgen05_gemm_matches_fp64(m, k):
    rng = np.random.default_rng(m + k)
    a = _bf16_bits(rng.normal(0, 1, (m, k)))
    b = _bf16_bits(rng.normal(0, 1, (256, k)))
    c = slide.gemm_bf16_nt(a, b)
    want = _bits_to_f64(a) @ _bits_to_f64(b).T
    # fp32 accumulation of k exact bf16 x bf16 products: |error| << k * 2^-24 * max|a| max|b|
    tol = 1e-6 * k * np.abs(_bits_to_f64(a)).max() * np.abs(_bits_to_f64(b)).max() + 1e-5
    assert np.abs(c - want).max() <= tol


def _model_params(width, seed):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.05, lo.num_params(width)).astype(np.float32)
    W1, b1, W2, b2, w3, b3 = lo.split(p, width)
    b1 += 0.05
    b2 += 0.05
    b3[:] = 4.0
    return p


def _batch(width, n, seed):
    tiles = instances.random_walks(width, n, (10, 80), seed=seed)
    slack = (np.arange(n) * 7 + seed) % 7
    target = np.random.default_rng(seed).uniform(0, 16, n)
    return tiles, slack.astype(np.int32), target.astype(np.float32)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(1e-30, np.linalg.norm(b)))


@pytest.mark.parametrize("width,n", [(4, 128), (5, 256)])
def test_gradients_match_fp64_restatement(gpu_solver, width, n):
    s = gpu_solver(width, "manhattan")
    p = _model_params(width, 11 + width)
    s.lbm_import(p)
    tiles, slack, target = _batch(width, n, 21 + width)
    loss, g = s.lbm_gradients(tiles, slack, target)
    want_loss, want_y, want_g = lo.forward_backward(p.astype(np.float64), tiles, slack, target, width)
    assert abs(loss - want_loss) <= 1e-4 * want_loss
    d = lo.feature_dim(width)
    offs = np.cumsum([0, d * 256, 256, 256 * 256, 256, 256, 1])
    names = ["W1", "b1", "W2", "b2", "w3", "b3"]
    for i, nm in enumerate(names):
        a, b = g[offs[i]:offs[i + 1]], want_g[offs[i]:offs[i + 1]]
        assert _rel(a, b) <= 2e-3, (nm, _rel(a, b))
    y = s.lbm_predict(tiles, slack)
    assert np.abs(y - want_y).max() <= 1e-3 * max(1.0, np.abs(want_y).max())


def test_predict_pads_ragged_batches(gpu_solver):
    s = gpu_solver(5, "manhattan")
    p = _model_params(5, 3)
    s.lbm_import(p)
    tiles, slack, _ = _batch(5, 200, 4)
    y_all = s.lbm_predict(tiles, slack)
    y_one = s.lbm_predict(tiles[:1], slack[:1])
    assert y_all.shape == (200,)
    assert abs(float(y_one[0]) - float(y_all[0])) <= 1e-5 * max(1.0, abs(float(y_all[0])))
    assert np.array_equal(s.lbm_export(), p)


def test_training_reduces_loss(gpu_solver):
    """A learnable target (2 x slack + Manhattan distance / 4) on a fixed batch."""
    w = 4
    s = gpu_solver(w, "manhattan")
    s.lbm_init(seed=7)
    tiles = instances.random_walks(w, 1024, (10, 60), seed=9)
    slack = (np.arange(1024) % 6).astype(np.int32)
    md = np.array([instances.manhattan(t, w) for t in tiles], dtype=np.float64)
    target = (2.0 * slack + md / 4.0).astype(np.float32)
    first = s.lbm_train_step(tiles, slack, target, 1e-3)
    for _ in range(60):
        last = s.lbm_train_step(tiles, slack, target, 1e-3)
    assert last < 0.25 * first, (first, last)


@pytest.mark.parametrize("loop", ["hybrid", "round", "persistent"])
def test_learned_lb_keeps_counts(gpu_solver, loop):
    """The model drives every root's predicted load -- in the round loop's
    plan and in the device loop's longest-first order and split -- and no
    count may change, whatever the (here untrained) model predicts."""
    s = gpu_solver(4, "manhattan")
    s.lbm_init(seed=5)
    states = instances.random_walks(4, 24, (60, 90), seed=21)
    want = oracle.solve(4, states, oracle.MD)
    extra = {"round": dict(persistent=0), "persistent": dict(persistent=1, handback_nodes=0)}.get(loop, {})
    s.set_config(lb_mode="learned", frontier_target=256, **extra)
    got = s.solve(states)
    for i, (a, b) in enumerate(zip(got, want)):
        assert_same(a, b, states[i], 4, "learned/%s/%d" % (loop, i))


def test_learned_lb_pdb24_golden(gpu_solver):
    g = load_golden("yama24_hard_new.json")["instances"][:6]
    states = np.array([x["tiles"] for x in g], dtype=np.uint8)
    s = gpu_solver(5, "pdb")
    s.lbm_init(seed=6)
    s.set_config(lb_mode="learned", frontier_target=1024)
    got = s.solve(states)
    for x, a, t in zip(g, got, states):
        assert (a["len"], a["nodes_total"]) == tuple(x["pdb"]), x["name"]
        assert slide.is_solution(t, a["moves"], 5)


def test_learned_lb_needs_a_model():
    s = slide.Solver(4, "manhattan", lb_mode="learned")
    with pytest.raises(slide.SlideError):
        s.solve(instances.random_walks(4, 2, 20, seed=1))
    s.close()


def test_trained_model_beats_the_slack_only_estimate(gpu_solver):
    """End to end through train_lb: labels from sp_dfs_round, GPU training,
    held-out evaluation.  The model's squared error on log2 subtree sizes
    must beat the best estimate that uses the slack alone (the mean per
    slack value), and rank roots well: the ordering the balancer needs."""
    import train_lb
    s = gpu_solver(4, "pdb")
    s.lbm_init(seed=3)
    tiles, slack, target, _ = train_lb.make_dataset(s, 40000, 5, 0x51, node_budget=2e9, log=lambda m: None)
    m = train_lb.train(s, tiles, slack, target, epochs=6, batch=2048, lr=2e-3, log=lambda m: None)
    assert m["mse"] < 0.9 * m["slack_only_mse"], m
    assert m["spearman"] > 0.6, m
