"""BF16 tensor-core MLP kernels against a float64 CPU oracle of the same network."""

import numpy as np
import pytest
import torch
from scipy.special import erf

from dendra_gb300 import _lib
from dendra_gb300.mlp import (EPI_BIAS, EPI_BIAS_GELU, EPI_GELU_GRAD, EPI_PLAIN, BF16MLP,
                              _gemm)

pytestmark = pytest.mark.gpu


def bf16(x):
    """Round float64/float32 values to bfloat16 (nearest even), returned as float64."""
    return torch.as_tensor(np.asarray(x, dtype=np.float32)).to(torch.bfloat16).double().numpy()


def gelu(z):
    return 0.5 * z * (1 + erf(z / np.sqrt(2)))


def gelu_grad(z):
    return 0.5 * (1 + erf(z / np.sqrt(2))) + z * np.exp(-0.5 * z * z) / np.sqrt(2 * np.pi)


def oracle_forward_backward(W16, b, x16, dy16):
    """float64 restatement with the kernels' bf16 roundings of activations and gradients."""
    hs, zs = [x16], []
    h = x16
    L = len(W16)
    for li in range(L):
        z = h @ W16[li] + b[li]
        zs.append(z)
        if li < L - 1:
            h = bf16(gelu(z))
            hs.append(h)
    dW, db = [None] * L, [None] * L
    dz = dy16
    for li in range(L - 1, -1, -1):
        dW[li] = hs[li].T @ dz
        db[li] = dz.sum(0)
        if li > 0:
            dz = bf16((dz @ W16[li].T) * gelu_grad(zs[li - 1]))
    return zs[-1], dW, db


@pytest.mark.parametrize("M", [300, 512])  # 300: mma.sync everywhere; 512: tcgen05 hidden layers
def test_forward_and_gradients_match_oracle(cuda, M):
    mlp = BF16MLP(device=cuda, seed=1)
    rng = np.random.default_rng(0)
    x = torch.as_tensor(rng.standard_normal((M, 4)), dtype=torch.float32)
    x16 = x.to(torch.bfloat16).to(cuda)
    y, acts, zs = mlp.forward(x16, keep=True)
    dy = torch.as_tensor(rng.standard_normal((M, 1)) * 0.1, dtype=torch.float32)
    dy16 = dy.to(torch.bfloat16).to(cuda)
    dW, db = mlp.backward(dy16, acts, zs)
    W16 = [w.double().cpu().numpy() for w in mlp.W16]
    b = [v.double().cpu().numpy() for v in mlp.b]
    y_ref, dW_ref, db_ref = oracle_forward_backward(W16, b, x16.double().cpu().numpy(),
                                                    dy16.double().cpu().numpy())
    np.testing.assert_allclose(y.double().cpu().numpy(), y_ref, rtol=2e-3, atol=2e-3)
    for li in range(len(W16)):
        scale = np.abs(dW_ref[li]).max()
        assert np.abs(dW[li].double().cpu().numpy() - dW_ref[li]).max() <= 3e-2 * scale, li
        np.testing.assert_allclose(db[li].double().cpu().numpy(), db_ref[li], rtol=3e-2,
                                   atol=3e-2 * np.abs(db_ref[li]).max())


def test_training_fits_a_smooth_function(cuda):
    """A few epochs on y = f(x) reduce the loss by an order of magnitude."""
    rng = np.random.default_rng(2)
    X = torch.as_tensor(rng.uniform(-1, 1, (16384, 4)), dtype=torch.float32)
    y = torch.sin(2 * X[:, 0]) + X[:, 1] * X[:, 2] - 0.5 * X[:, 3] ** 2
    mlp = BF16MLP(device=cuda, seed=3)
    losses = mlp.train(X, y, epochs=12, batch=1024, lr=2e-3)
    assert losses[-1] < 0.1 * losses[0]
    pred = mlp.predict(X[:2048])
    err = (pred.cpu() - y[:2048]).abs().mean()
    assert float(err) < 0.08


@pytest.mark.parametrize("K", [64, 128, 256])
@pytest.mark.parametrize("N", [256, 512])
def test_tcgen05_gemm_matches_float64_and_the_mma_sync_path(cuda, K, N):
    """K-major operands run on tcgen05 (TMA + TMEM); the same product with B
    addressed N-major runs on mma.sync.  Both against a float64 product."""
    L = _lib.load()
    rng = np.random.default_rng(K + N)
    M = 384
    A = torch.as_tensor(rng.standard_normal((M, K)), dtype=torch.float32).to(torch.bfloat16).to(cuda)
    W = torch.as_tensor(rng.standard_normal((K, N)) / np.sqrt(K),
                        dtype=torch.float32).to(torch.bfloat16).to(cuda)
    Wt = W.t().contiguous()
    bias = torch.as_tensor(rng.standard_normal(N), dtype=torch.float32).to(cuda)
    aux = torch.as_tensor(rng.standard_normal((M, N)), dtype=torch.float32).to(cuda)
    assert L.dgb_mlp_gemm_path(M, N, K, A.data_ptr(), K, 1, Wt.data_ptr(), 1, K) == 1
    assert L.dgb_mlp_gemm_path(M, N, K, A.data_ptr(), K, 1, W.data_ptr(), N, 1) == 0
    acc = A.double().cpu().numpy() @ W.double().cpu().numpy()
    z = acc + bias.double().cpu().numpy()
    ref = {EPI_PLAIN: (acc, None), EPI_BIAS: (z, None), EPI_BIAS_GELU: (z, bf16(gelu(z))),
           EPI_GELU_GRAD: (acc * gelu_grad(aux.double().cpu().numpy()),
                           bf16(acc * gelu_grad(aux.double().cpu().numpy())))}
    for epi, (r32, r16) in ref.items():
        outs = []
        for B, sbk, sbn in ((Wt, 1, K), (W, N, 1)):
            o32 = torch.full((M, N), float("nan"), dtype=torch.float32, device=cuda)
            o16 = torch.zeros((M, N), dtype=torch.bfloat16, device=cuda)
            _gemm(M, N, K, A, K, 1, B, sbk, sbn, bias=bias if epi in (EPI_BIAS, EPI_BIAS_GELU)
                  else None, epi=epi, aux=aux if epi == EPI_GELU_GRAD else None, out32=o32,
                  out16=o16)
            outs.append((o32.double().cpu().numpy(), o16.double().cpu().numpy()))
        assert L.dgb_mlp_gemm_status(None) == 0
        scale = np.abs(r32).max()
        for o32, o16 in outs:  # tcgen05, then mma.sync
            np.testing.assert_allclose(o32, r32, rtol=0, atol=2e-5 * scale, err_msg=str(epi))
            if r16 is not None:
                np.testing.assert_allclose(o16, r16, rtol=1e-2, atol=1e-2 * scale)
        np.testing.assert_allclose(outs[0][0], outs[1][0], rtol=0, atol=2e-5 * scale)


def test_tcgen05_load_wait_timeout_surfaces(cuda):
    """A TMA load wait limited to zero polls gives up at once: the kernel drains
    its copies, frees its tensor memory and flags the error; the status call
    raises DgbTimeout, and with the default limit restored the same GEMM runs
    correctly on the same context.  Nothing faults or hangs: every wait is
    bounded and the copies are real, in-bounds TMA loads."""
    from dendra_gb300.mlp import gemm_status

    L = _lib.load()
    rng = np.random.default_rng(3)
    M, N, K = 128, 256, 256
    A = torch.as_tensor(rng.standard_normal((M, K)), dtype=torch.float32).to(torch.bfloat16).to(cuda)
    Wt = torch.as_tensor(rng.standard_normal((N, K)) / 16, dtype=torch.float32).to(
        torch.bfloat16).to(cuda)
    assert L.dgb_mlp_gemm_path(M, N, K, A.data_ptr(), K, 1, Wt.data_ptr(), 1, K) == 1
    o32 = torch.zeros((M, N), dtype=torch.float32, device=cuda)
    try:
        assert L.dgb_mlp_gemm_set_wait_limit(0) == 0
        _gemm(M, N, K, A, K, 1, Wt, 1, K, epi=EPI_PLAIN, out32=o32)
        with pytest.raises(_lib.DgbTimeout, match="still usable"):
            gemm_status(cuda)
    finally:
        assert L.dgb_mlp_gemm_set_wait_limit(-1) == 0
    _gemm(M, N, K, A, K, 1, Wt, 1, K, epi=EPI_PLAIN, out32=o32)
    gemm_status(cuda)
    ref = A.double().cpu().numpy() @ Wt.double().cpu().numpy().T
    np.testing.assert_allclose(o32.double().cpu().numpy(), ref, rtol=0,
                               atol=2e-5 * np.abs(ref).max())
