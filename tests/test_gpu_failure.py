"""Failure handling on the GPU without a fault: a device wait that nothing
satisfies ends after its limit with SP_ERR_TIMEOUT, and the solver (and the
CUDA context) keep working."""
import time

import pytest

import instances
import oracle
from test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("heuristic", ["manhattan", "pdb"])
def test_stalled_pool_times_out_and_solver_recovers(gpu_solver, heuristic):
    s = gpu_solver(4, heuristic)
    t0 = time.perf_counter()
    status = s.selftest_stall(200)
    dt = time.perf_counter() - t0
    assert status == -8  # SP_ERR_TIMEOUT
    assert 0.15 <= dt < 10.0
    states = instances.random_walks(4, 6, (30, 50), seed=12)
    tabs = oracle.tables(4) if heuristic == "pdb" else None
    want = oracle.solve(4, states, oracle.PDB if tabs else oracle.MD, tabs)
    for i, (a, b) in enumerate(zip(s.solve(states), want)):
        assert_same(a, b, states[i], 4, "after-stall/%d" % i)


@pytest.mark.parametrize("chunk", [0, 1, 2, 3])
def test_tensor_core_gemm_wait_runs_out_and_next_gemm_is_exact(chunk):
    """The learned balancer's tcgen05 GEMM with one K chunk never copied in:
    the wait for it ends after its 50 ms limit with SP_ERR_TIMEOUT (copies in
    flight drained, tensor memory freed), and the next GEMM on the same
    context is exact against an FP64 product of the same bf16 inputs, which
    it could not be if the stalled CTA had kept its tensor memory."""
    import numpy as np
    import torch
    import slide
    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    assert slide.selftest_gemm_stall(chunk, 50) == -8  # SP_ERR_TIMEOUT
    assert time.perf_counter() - t0 < 10.0
    rng = np.random.default_rng(chunk)
    a = torch.from_numpy(rng.standard_normal((256, 192)).astype(np.float32)).to(torch.bfloat16)
    b = torch.from_numpy(rng.standard_normal((256, 192)).astype(np.float32)).to(torch.bfloat16)
    c = slide.gemm_bf16_nt(a.view(torch.int16).numpy().view(np.uint16), b.view(torch.int16).numpy().view(np.uint16))
    want = a.double().numpy() @ b.double().numpy().T
    assert np.abs(c - want).max() <= 1e-6 * 192 * float(a.abs().max()) * float(b.abs().max())
