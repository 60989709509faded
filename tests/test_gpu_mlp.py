"""The tensor-core GEMM and the surrogate network's forward, backward and Adam steps on the GPU,
through the C ABI, against the CPU restatement in oracle/mlp_oracle.py."""
import os
import sys

import numpy as np
import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu
sys.path.insert(0, os.path.join(REPO, "oracle"))
import mlp_oracle as M  # noqa: E402

N_IN, WIDTH, N_OUT = 64, 256, 132


def _torch():
    return pytest.importorskip("torch")


@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (200, 256, 300), (1000, 144, 256), (64, 64, 8),
                                   (300, 100, 1000), (129, 257, 72)])
def test_gemm_matches_numpy(m, n, k):
    torch = _torch()
    from souffle_gb300 import gpu
    g = torch.Generator().manual_seed(m * 7 + n + k)
    a = torch.randn(m, k, generator=g).cuda()
    b = torch.randn(n, k, generator=g).cuda()
    c = torch.full((m, n), float("nan"), device="cuda")
    gpu.gemm_bf16(a.data_ptr(), b.data_ptr(), m, n, k, c.data_ptr())
    torch.cuda.synchronize()
    ab, bb = M.bf16(a.cpu().numpy()).astype(np.float64), M.bf16(b.cpu().numpy()).astype(np.float64)
    ref = ab @ bb.T
    scale = np.abs(ab) @ np.abs(bb).T
    err = np.abs(c.cpu().numpy() - ref)
    assert np.all(np.isfinite(c.cpu().numpy()))
    assert np.all(err <= (k * 1.2e-7 + 1e-6) * scale + 1e-30), err.max()


def _setup(m, seed, width=WIDTH):
    torch = _torch()
    from souffle_gb300 import gpu
    net = gpu.Mlp(N_IN, N_OUT, max_batch=1024, seed=seed, width=width)
    rng = np.random.default_rng(seed)
    x = rng.normal(0, 1, (m, N_IN)).astype(np.float32)
    t = rng.normal(0, 0.5, (m, N_OUT)).astype(np.float32)
    return torch, net, x, t


@pytest.mark.parametrize("width", [128, 256])
@pytest.mark.parametrize("m", [128, 300])
def test_forward_matches_oracle(m, width):
    torch, net, x, _ = _setup(m, 3, width)
    p = net.get_params()
    xd = torch.from_numpy(x).cuda()
    y = torch.empty(m, N_OUT, device="cuda")
    net.forward(xd.data_ptr(), m, y.data_ptr())
    torch.cuda.synchronize()
    ref = M.forward(p, x, N_IN, width, N_OUT, emulate=True)
    err = np.abs(y.cpu().numpy() - ref).max()
    assert err <= 2e-2 * np.abs(ref).max(), err


@pytest.mark.parametrize("width", [128, 256])
@pytest.mark.parametrize("m", [128, 300])
def test_gradients_match_oracle(m, width):
    torch, net, x, t = _setup(m, 5, width)
    p = net.get_params()
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    loss, g = net.gradients(xd.data_ptr(), td.data_ptr(), m)
    ref_loss, ref_g = M.loss_and_grads(p, x, t, N_IN, width, N_OUT, emulate=True)
    assert loss == pytest.approx(ref_loss, rel=1e-4)
    k = 0
    for (ws, bs) in M.shapes(N_IN, width, N_OUT):
        for size in (ws[0] * ws[1], bs[0]):
            a, b = g[k:k + size], ref_g[k:k + size]
            assert np.linalg.norm(a - b) <= 1e-2 * np.linalg.norm(b) + 1e-12, (k, size)
            k += size
    assert np.array_equal(net.get_params(), p)       # gradients leave the parameters alone


def test_training_fits_a_smooth_map():
    torch, net, _, _ = _setup(512, 7)
    rng = np.random.default_rng(8)
    R = rng.normal(0, 0.3, (N_IN, N_OUT)).astype(np.float32)
    x = rng.normal(0, 1, (512, N_IN)).astype(np.float32)
    t = np.sin(x @ R).astype(np.float32)
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    first = net.train_step(xd.data_ptr(), td.data_ptr(), 512, 1e-3)
    for _ in range(300):
        last = net.train_step(xd.data_ptr(), td.data_ptr(), 512, 1e-3)
    assert last < 0.2 * first, (first, last)
    y = torch.empty(512, N_OUT, device="cuda")
    net.forward(xd.data_ptr(), 512, y.data_ptr())
    torch.cuda.synchronize()
    assert np.mean((y.cpu().numpy() - t) ** 2) == pytest.approx(last, rel=0.3)


@pytest.mark.parametrize("width", [128, 256])
@pytest.mark.parametrize("m", [1, 129, 300, 152 * 128 * 3 + 77])
def test_fused_forward_matches_oracle_and_layered(m, width):
    """The one-kernel forward (activations on chip, SiLU from a hardware tanh) against the CPU
    restatement, and against the per-layer GEMMs: both round to BF16 at the same points, so they
    differ only where the SiLU approximations put a value on the other side of a BF16 rounding
    boundary.  The largest case gives every CTA several tiles and an odd tile count; both hidden
    widths the kernel supports."""
    torch = _torch()
    from souffle_gb300 import gpu
    gpu_net = gpu.Mlp(N_IN, N_OUT, max_batch=max(m, 1024), seed=11, width=width)
    rng = np.random.default_rng(m)
    x = rng.normal(0, 1, (m, N_IN)).astype(np.float32)
    p = gpu_net.get_params()
    xd = torch.from_numpy(x).cuda()
    y = torch.full((m, N_OUT), float("nan"), device="cuda")
    yl = torch.full((m, N_OUT), float("nan"), device="cuda")
    gpu_net.forward(xd.data_ptr(), m, y.data_ptr())
    gpu_net.forward_layered(xd.data_ptr(), m, yl.data_ptr())
    torch.cuda.synchronize()
    yf, yl = y.cpu().numpy(), yl.cpu().numpy()
    assert np.all(np.isfinite(yf))
    rows = np.arange(m) if m <= 2048 else np.random.default_rng(1).choice(m, 2048, replace=False)
    ref = M.forward(p, x[rows], N_IN, width, N_OUT, emulate=True)
    assert np.abs(yf[rows] - ref).max() <= 2e-2 * np.abs(ref).max()
    # fused against layered: RMS of the difference within 1 % of the RMS output
    assert np.sqrt(np.mean((yf - yl) ** 2)) <= 1e-2 * np.sqrt(np.mean(yl ** 2))
    # same input, same bits
    y2 = torch.empty_like(y)
    gpu_net.forward(xd.data_ptr(), m, y2.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(y2.cpu().numpy(), yf)
