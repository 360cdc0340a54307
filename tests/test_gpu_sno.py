"""GPU tests of the spectral neural operator surrogate (pyofsschanged_gb300.surrogate).

* the BF16 tensor-core GEMM against torch on the same BF16 operands (all
  transposes, batch strides, split-K, fused epilogues);
* the network's forward pass and every parameter gradient against the CPU
  restatement oracle/sno_oracle.py (same BF16 rounding points);
* training on the engine's own propagations gains over the method without the
  network (linear propagation only);
* the fallback: members above the error tolerance get the RK4IP engine's output.
"""

import numpy as np
import pytest
import torch

from oracle import sno_oracle as so
from pyofsschanged_gb300 import surrogate as sg

pytestmark = pytest.mark.gpu


def _bf(x):
    return x.to(torch.bfloat16)


@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_gemm_matches_torch(cuda_ready, ta, tb):
    torch.manual_seed(0)
    dev = torch.device("cuda")
    for (M, N, K, batch) in [(64, 64, 32, 1), (100, 70, 45, 3), (7, 130, 300, 2), (256, 2, 17, 1)]:
        A = _bf(torch.randn(batch, K, M, device=dev) if ta else torch.randn(batch, M, K, device=dev))
        B = _bf(torch.randn(batch, N, K, device=dev) if tb else torch.randn(batch, K, N, device=dev))
        C0 = torch.randn(batch, M, N, device=dev)
        bias = torch.randn(N, device=dev)
        C = C0.clone()
        g16 = torch.empty(batch, M, N, dtype=torch.bfloat16, device=dev)
        sg.gemm(M, N, K, A, B, C, ta=ta, tb=tb, sA=A[0].numel(), sB=B[0].numel(), sC=M * N, batch=batch,
                alpha=0.5, beta=2.0, bias=bias, gelu_out=g16, sO=M * N)
        a = A.float().transpose(1, 2) if ta else A.float()
        b = B.float().transpose(1, 2) if tb else B.float()
        ref = 0.5 * torch.bmm(a, b) + 2.0 * C0 + bias
        torch.cuda.synchronize()
        assert torch.allclose(C, ref, rtol=1e-4, atol=1e-4 * K ** 0.5), (M, N, K, (C - ref).abs().max())
        gel = 0.5 * ref * (1 + torch.tanh(0.7978845608028654 * (ref + 0.044715 * ref ** 3)))
        assert torch.allclose(g16.float(), gel, rtol=1e-2, atol=1e-2)
        # split-K accumulation into C
        C2 = C0.clone()
        sg.gemm(M, N, K, A, B, C2, ta=ta, tb=tb, sA=A[0].numel(), sB=B[0].numel(), sC=M * N, batch=batch,
                beta=1.0, splits=3)
        assert torch.allclose(C2, torch.bmm(a, b) + C0, rtol=1e-4, atol=1e-4 * K ** 0.5)
    assert sg.gemm_timeouts() == 0


def test_forward_and_gradients_match_oracle(cuda_ready):
    n, cin, W, K, L, H, B = 256, 4, 16, 8, 2, 12, 3
    rng = np.random.default_rng(3)
    p = so.init_params(cin, W, K, L, H, rng)
    for k in p:
        if k.startswith("b"):
            p[k] = 0.1 * rng.standard_normal(p[k].shape)
    p["Q2"] = rng.standard_normal(p["Q2"].shape) * 0.3
    feat = so.bf16(rng.standard_normal((B, n, cin)))
    resid = rng.standard_normal((B, n, 2)).astype(np.float32).astype(np.float64)
    target = resid + 0.5 * rng.standard_normal((B, n, 2)).astype(np.float32)
    F, G = so.dft_mats(n, K)
    out_ref, cache = so.forward(p, feat, resid, F, G)
    err_ref, dout_ref = so.loss(out_ref, target)
    g_ref = so.backward(p, cache, dout_ref, F, G)

    net = sg.SpectralNeuralOperator(n=n, width=W, modes=K, layers=L, hidden=H, params=p)
    dev = net.dev
    feat16 = torch.tensor(feat.reshape(B * n, cin), dtype=torch.float32, device=dev).to(torch.bfloat16)
    res = torch.tensor(resid.reshape(B * n, 2), dtype=torch.float32, device=dev)
    tgt = torch.tensor(target.reshape(B * n, 2), dtype=torch.float32, device=dev)
    out = net.forward(feat16, res)
    grad = torch.empty_like(out)
    err = net.loss(out, tgt, grad)
    g = net.backward(grad)
    torch.cuda.synchronize()

    def rel(a, b):
        return np.linalg.norm(np.asarray(a, float) - b) / max(np.linalg.norm(b), 1e-30)

    assert rel(out.cpu().numpy().reshape(B, n, 2), out_ref) < 2e-3
    np.testing.assert_allclose(err.cpu().numpy(), err_ref, rtol=1e-2)
    for k in p:
        assert rel(g[k].cpu().numpy(), g_ref[k]) < 2e-2, (k, rel(g[k].cpu().numpy(), g_ref[k]))


@pytest.fixture(scope="module")
def short_segment():
    """Engine propagations through a 5 mm segment (a mild nonlinear change)."""
    z = 5e-6
    params, A0 = sg.sample_pulses(72, seed=11, power_kw=(1.0, 5.0))
    AL, st = sg.propagate(A0, z)
    assert all(s["status"] == 0 for s in st)
    return z, A0, AL


def test_training_gains_over_linear_propagation(cuda_ready, short_segment):
    z, A0, AL = short_segment
    pic, a0, aL, _ = sg.make_dataset(A0, AL, z)
    tr, te = slice(0, 56), slice(56, 72)
    net = sg.SpectralNeuralOperator(width=32, modes=32, layers=2, hidden=64, seed=0)
    hist = sg.train(net, pic, a0[tr], aL[tr], epochs=25, batch=8, lr=3e-3)
    assert hist[-1] < 0.5 * hist[0]
    base = sg.rel_err(a0[te], aL[te])             # linear propagation alone
    pred = sg.rel_err(sg.predict(net, pic, a0[te]), aL[te])
    assert np.median(pred) < 0.5 * np.median(base), (np.median(pred), np.median(base))


def test_fallback_uses_the_engine(cuda_ready, short_segment):
    z, A0, AL = short_segment
    pic = sg.Picture()
    nets = [sg.SpectralNeuralOperator(width=16, modes=8, layers=1, hidden=16, seed=s) for s in (0, 1)]
    sur = sg.SurrogateWithFallback(nets, pic, tol=-1.0)  # a negative tolerance rejects every member
    out, accept, est = sur(A0[:4], z)
    assert not accept.any()
    ref, _ = sg.propagate(A0[:4], z)
    np.testing.assert_array_equal(out, ref)  # the engine's own result, bit for bit
    sur.tol = np.inf
    out2, accept2, _ = sur(A0[:4], z)
    assert accept2.all()
    A0t = torch.as_tensor(A0[:4], dtype=torch.complex128, device=pic.dev)
    scale = A0t.abs().amax(dim=1, keepdim=True)
    mean, _ = sur.estimate(A0t / scale)
    np.testing.assert_allclose(out2, (pic.from_ip(mean, z) * scale).cpu().numpy(), rtol=1e-12, atol=1e-9)
