"""Tensor-core (tcgen05) path of the surrogate: the GEMM kernel against an
FP64 product of the same BF16 operands, the MLP gradients against the FP64
numpy oracle (oracle/mlp64.py, with BF16 rounding at the same storage points),
and that training on the GPU lowers the loss."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GEMM_RTOL = 2e-3      # fp32 accumulation of exact bf16 products
GRAD_RTOL = 3e-2      # relative L2 error of the whole gradient vector


@pytest.fixture(scope="module")
def sur():
    from ismc_gb300 import build
    from ismc_gb300.surrogate import Surrogate
    build.build()
    s = Surrogate(0, max_batch=4096, seed=3)
    yield s
    s.close()


@pytest.mark.parametrize("M,N,K,splits", [(128, 256, 64, 1), (256, 256, 256, 1), (512, 16, 256, 1),
                                          (256, 64, 4096, 16), (128, 256, 4096, 16),
                                          (4096, 256, 256, 1),
                                          # deep K: stages refilled while the MMAs run
                                          (256, 64, 1024, 1), (512, 16, 1280, 1),
                                          (128, 256, 1024, 2)])
def test_umma_gemm_matches_fp64(sur, M, N, K, splits):
    import torch
    g = torch.Generator().manual_seed(M * 7 + N + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, generator=g).to(torch.bfloat16)
    dA, dB = A.cuda(), B.cuda()
    D = torch.empty(M, N, device="cuda", dtype=torch.float32)
    rc = sur.lib.ismc_mlp_gemm_test(sur.h, dA.data_ptr(), dB.data_ptr(), D.data_ptr(), M, N, K, splits)
    assert rc == 0, sur._err(sur.h)
    ref = A.double() @ B.double().T
    err = (D.cpu().double() - ref).abs().max().item()
    scale = ref.abs().max().item()
    assert err <= GEMM_RTOL * scale, (err, scale)


@pytest.mark.parametrize("B", [512, 4096])      # 4096: the training batch's split-K choices
def test_mlp_gradients_vs_fp64_oracle(sur, B):
    from oracle import mlp64
    rng = np.random.default_rng(0)
    x = mlp64.LO + (mlp64.HI - mlp64.LO) * rng.random((B, 5))
    y = rng.random((B, 3)) * [0.5, 0.3, 0.2]
    p = sur.get_params().astype(np.float64)
    loss, g = sur.grad(x.astype(np.float32), y.astype(np.float32))
    # the oracle sees the same fp32 inputs
    x32, y32 = x.astype(np.float32).astype(np.float64), y.astype(np.float32).astype(np.float64)
    loss64, g64 = mlp64.loss_and_grad(p, x32, y32, bf16_emulation=True)
    assert abs(loss - loss64) <= 1e-3 * abs(loss64) + 1e-4, (loss, loss64)
    rel = np.linalg.norm(g - g64) / np.linalg.norm(g64)
    assert rel < GRAD_RTOL, rel
    # and against the exact FP64 network (no bf16): agreement at bf16 resolution
    _, g_exact = mlp64.loss_and_grad(p, x32, y32, bf16_emulation=False)
    assert np.dot(g, g_exact) / (np.linalg.norm(g) * np.linalg.norm(g_exact)) > 0.99


def test_mlp_forward_matches_oracle(sur):
    from oracle import mlp64
    rng = np.random.default_rng(1)
    x = mlp64.LO + (mlp64.HI - mlp64.LO) * rng.random((300, 5))      # pads to 384 internally
    out = sur.forward(x.astype(np.float32)).cpu().numpy()
    ref, _, _ = mlp64.forward(sur.get_params().astype(np.float64),
                              x.astype(np.float32).astype(np.float64), mlp64.bf16)
    assert np.max(np.abs(out - ref[:, :6])) < 2e-2 * max(1.0, np.max(np.abs(ref)))


def test_adam_trajectory_tracks_fp64_oracle():
    """20 Adam steps on the GPU move the parameters the way 20 FP64 Adam steps
    on the oracle's gradients (with bf16 emulation) do."""
    import torch
    from oracle import mlp64
    from ismc_gb300.surrogate import Surrogate
    s = Surrogate(0, max_batch=512, seed=21)
    try:
        rng = np.random.default_rng(7)
        x = (mlp64.LO + (mlp64.HI - mlp64.LO) * rng.random((512, 5))).astype(np.float32)
        y = (rng.random((512, 3)) * [0.5, 0.3, 0.2]).astype(np.float32)
        dx, dy = torch.as_tensor(x).cuda(), torch.as_tensor(y).cuda()
        p0 = s.get_params().astype(np.float64)
        lr, steps = 1e-3, 20
        for _ in range(steps):
            s.train_step(dx, dy, lr)
        p_gpu = s.get_params().astype(np.float64)
        p, m, v = p0.copy(), np.zeros_like(p0), np.zeros_like(p0)
        x64, y64 = x.astype(np.float64), y.astype(np.float64)
        for t in range(1, steps + 1):
            _, g = mlp64.loss_and_grad(p.astype(np.float32).astype(np.float64), x64, y64,
                                       bf16_emulation=True)
            m = 0.9 * m + 0.1 * g
            v = 0.999 * v + 0.001 * g * g
            p = p - lr * (m / (1 - 0.9 ** t)) / (np.sqrt(v / (1 - 0.999 ** t)) + 1e-8)
        du_gpu, du_ref = p_gpu - p0, p - p0
        rel = np.linalg.norm(du_gpu - du_ref) / np.linalg.norm(du_ref)
        assert rel < 0.1, rel
    finally:
        s.close()


def test_mlp_training_lowers_loss():
    """Fit a smooth synthetic map (stand-in targets; the Monte Carlo data path is
    exercised by the surrogate-solve test): the loss must fall well below its start."""
    import torch
    from ismc_gb300.surrogate import LO, HI, Surrogate
    s = Surrogate(0, max_batch=4096, seed=11)
    try:
        rng = np.random.default_rng(5)
        X = LO + (HI - LO) * rng.random((32768, 5))
        u = (X - LO) / (HI - LO)
        Y = np.stack([0.5 * np.exp(-2 * u[:, 0]) * (0.3 + u[:, 1]), 0.3 * u[:, 3] * (1 - u[:, 0]),
                      0.2 * np.exp(-3 * u[:, 1] * u[:, 3])], 1)
        Y = Y + 0.002 * rng.standard_normal(Y.shape)
        hist = s.train(X.astype(np.float32), Y.astype(np.float32), epochs=12, batch=4096, lr=1e-3)
        assert hist[-1] < hist[0] - 2.0, hist
        pred = s.forward(X[:4096].astype(np.float32)).cpu().numpy()[:, :3]
        assert np.sqrt(np.mean((pred - Y[:4096]) ** 2)) < 0.02
    finally:
        s.close()


def test_pipeline_wait_limit_runs_out_and_context_recovers(sur):
    """With the wait limit at 0 every product's first pipeline wait gives up at
    once: the forward pass returns ISMC_ERR_INTERNAL (after each block let its
    requested tiles land and freed its TMEM).  With the limit restored, the
    same context computes the same outputs as before."""
    from ismc_gb300 import IsmcError, _abi
    from oracle import mlp64
    rng = np.random.default_rng(5)
    x = (mlp64.LO + (mlp64.HI - mlp64.LO) * rng.random((256, 5))).astype(np.float32)
    before = sur.forward(x).cpu().numpy()
    assert sur.lib.ismc_mlp_set_wait_limit(sur.h, 0) == 0
    try:
        with pytest.raises(IsmcError) as e:
            sur.forward(x)
        assert e.value.code == _abi.ERR_INTERNAL
        assert "timed out" in str(e.value)
    finally:
        assert sur.lib.ismc_mlp_set_wait_limit(sur.h, 1 << 22) == 0
    after = sur.forward(x).cpu().numpy()
    assert np.array_equal(before, after)
