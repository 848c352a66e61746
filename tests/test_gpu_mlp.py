"""The learned initialiser's tensor-core kernels against references:
  * the tcgen05 GEMM against an FP32 matmul of the same bf16 operands
    (|err| <= 1e-5 sqrt(K) max|A| max|B|: both accumulate in FP32 in
    different orders);
  * forward outputs and every layer's weight and bias gradients against the
    CPU oracle with the library's bf16 rounding points (norm-wise relative
    error <= 2e-2; single bf16 roundings may land on the other side where
    accumulation orders differ);
  * Adam training lowers the loss on a learnable task."""
import numpy as np
import pytest
import torch

from oracle.mlp_oracle import MlpOracle, bf16, init_params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(300, 256, 288), (4096, 16, 256), (256, 288, 4096),
                                   (1000, 256, 16), (12, 256, 4096), (129, 12, 64)])
def test_umma_gemm_matches_fp32_matmul(built, cuda, M, N, K):
    from cudimot_gb300 import mlp
    g = torch.Generator(device="cpu").manual_seed(M * 7 + N + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).to(cuda)
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).to(cuda)
    got = mlp.gemm_bf16(A, B)
    torch.cuda.synchronize()
    ref = A.float() @ B.float().T
    tol = 1e-5 * np.sqrt(K) * A.float().abs().max().item() * B.float().abs().max().item()
    err = (got - ref).abs().max().item()
    assert err <= tol, (err, tol)


def _net(seed=1):
    from cudimot_gb300 import mlp
    cfg = mlp.default_cfg()
    W, b = init_params(cfg.n_in, cfg.hidden, cfg.n_mu + cfg.n_sig, seed=seed)
    rng = np.random.default_rng(seed)
    W[3] *= 5.0
    b = [(rng.standard_normal(x.shape) * 0.05).astype(np.float32) for x in b]
    net = mlp.Mlp(cfg)
    net.set_params(W, b)
    o = MlpOracle(W, b, cfg.n_mu, cfg.n_sig, list(cfg.group)[:cfg.n_mu])
    return cfg, net, o


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def test_forward_matches_oracle(built, cuda):
    cfg, net, o = _net()
    rng = np.random.default_rng(3)
    x = bf16(rng.uniform(0.0, 1.2, (640, cfg.n_in)).astype(np.float32))
    xt = torch.as_tensor(x).to(torch.bfloat16).to(cuda)
    out = net.forward(xt)
    torch.cuda.synchronize()
    net.check()
    ref, _, _ = o.forward(x)
    got = out.cpu().numpy()[:, :cfg.n_mu + cfg.n_sig]
    assert _rel(got, ref) < 2e-2, _rel(got, ref)
    assert np.all(out.cpu().numpy()[:, cfg.n_mu + cfg.n_sig:] == 0)


def test_gradients_match_oracle(built, cuda):
    cfg, net, o = _net(seed=5)
    rng = np.random.default_rng(6)
    B = 512
    x = bf16(rng.uniform(0.0, 1.2, (B, cfg.n_in)).astype(np.float32))
    t = rng.standard_normal((B, cfg.n_mu)).astype(np.float32)
    loss = torch.zeros(1, dtype=torch.float32, device=cuda)
    net.gradients(torch.as_tensor(x).to(torch.bfloat16).to(cuda), torch.as_tensor(t).to(cuda), loss)
    torch.cuda.synchronize()
    net.check()
    _, _, gW, gb = net.get_params(grads=True)
    rl, dW, db = o.gradients(x, t)
    assert abs(loss.item() - rl) <= 2e-2 * abs(rl)
    for l in range(4):
        assert _rel(gW[l], dW[l]) < 3e-2, (l, _rel(gW[l], dW[l]))
        assert _rel(gb[l], db[l]) < 3e-2, (l, _rel(gb[l], db[l]))


def test_adam_training_lowers_loss(built, cuda):
    cfg, net, _ = _net(seed=9)
    rng = np.random.default_rng(10)
    B = 1024
    P = rng.standard_normal((cfg.n_in, cfg.n_mu)).astype(np.float32) / np.sqrt(cfg.n_in)
    x = rng.uniform(0.0, 1.0, (B * 8, cfg.n_in)).astype(np.float32)
    t = np.tanh(x @ P * 3.0).astype(np.float32)
    xt = torch.as_tensor(x).to(torch.bfloat16).to(cuda)
    tt = torch.as_tensor(t).to(cuda)
    loss = torch.zeros(1, dtype=torch.float32, device=cuda)
    hist = []
    for step in range(300):
        k = step % 8
        net.train_step(xt[k * B:(k + 1) * B], tt[k * B:(k + 1) * B], loss)
        if step % 50 == 0 or step == 299:
            torch.cuda.synchronize()
            hist.append(loss.item())
    net.check()
    assert np.isfinite(hist).all()
    assert hist[-1] < hist[0] - 2.0, hist


@pytest.mark.parametrize("layer,n", [(0, 300), (1, 262144 + 77)])
def test_hidden_layer_matches_reference(built, cuda, layer, n):
    """One inference hidden layer (the persistent tcgen05 kernel: one CTA
    per SM looping over 128-row tiles, two TMEM accumulators) against an
    FP32 matmul of the same bf16 operands with the library's rounding
    points: z = bf16(x W^T + b), out = bf16(gelu(z)). 262,221 rows give
    2,049 tiles, so every CTA runs many tiles and the last one is ragged.
    A z that lands on the other side of a bf16 rounding (different
    accumulation order) moves its output by one bf16 step: the bound is two
    steps plus a small absolute term near zero."""
    from oracle.mlp_oracle import gelu
    cfg, net, _ = _net(seed=2)
    W, b, _, _ = net.get_params(grads=True)
    g = torch.Generator(device="cpu").manual_seed(n + layer)
    width = cfg.n_in if layer == 0 else cfg.hidden
    x = (torch.rand(n, width, generator=g) * 1.2).to(torch.bfloat16).to(cuda)
    out = torch.full((n, cfg.hidden), float("nan"), dtype=torch.bfloat16, device=cuda)
    net.hidden_layer(layer, x, out)
    torch.cuda.synchronize()
    net.check()
    w = torch.as_tensor(bf16(W[layer])).to(cuda)
    z = (x.float() @ w.T + torch.as_tensor(b[layer]).to(cuda)).to(torch.bfloat16).float()
    ref = torch.as_tensor(gelu(z.cpu().numpy().astype(np.float64))).to(torch.bfloat16).float()
    got = out.float().cpu()
    assert torch.isfinite(got).all()
    err = (got - ref).abs()
    assert bool((err <= 2.0 ** -6 * ref.abs() + 2e-3).all()), float(err.max())
