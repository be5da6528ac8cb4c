"""The training loss kernel (ubs.loss, fused_ssim drop-in) against the FP64
oracle (itself pinned to the reference's utils/loss_utils.py SSIM) and a plain
PyTorch FP32 SSIM of the same definition.

Tolerances: loss values 2e-6 absolute (FP32 sums over up to 6M points, the
oracle in FP64); gradients 1e-4 of the gradient's largest magnitude (the
SSIM gradient is a difference of windowed terms ~1/C2 that cancel in flat
regions, as in any FP32 implementation: the reference's own FP32 SSIM sits
5e-6 from FP64 on the golden cases)."""
import numpy as np
import pytest
import torch
import torch.nn.functional as F

import oracle as orc
from ubs import loss as LS

pytestmark = pytest.mark.gpu
DEV = "cuda"


def images(shape, seed, near=False):
    g = torch.Generator().manual_seed(seed)
    gt = torch.rand(*shape, generator=g)
    img = (gt + 0.05 * torch.randn(*shape, generator=g)).clamp(0, 1) if near else \
        torch.rand(*shape, generator=g)
    return img, gt


def rel_max(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).max() / max(np.abs(b).max(), 1e-30))


def torch_ssim(x, y):
    """utils/loss_utils.py's SSIM in FP32 PyTorch (conv2d, zero padding)."""
    c = x.shape[1]
    d = torch.arange(11, dtype=torch.float64) - 5
    g = torch.exp(-d * d / (2 * 1.5 ** 2))
    g = (g / g.sum()).float()
    win = (g[:, None] @ g[None, :]).expand(c, 1, 11, 11).contiguous().to(x.device)
    conv = lambda a: F.conv2d(a, win, padding=5, groups=c)  # noqa: E731
    mu1, mu2 = conv(x), conv(y)
    s1, s2, s12 = conv(x * x) - mu1 ** 2, conv(y * y) - mu2 ** 2, conv(x * y) - mu1 * mu2
    C1, C2 = 0.01 ** 2, 0.03 ** 2
    m = ((2 * mu1 * mu2 + C1) * (2 * s12 + C2)) / ((mu1 ** 2 + mu2 ** 2 + C1) * (s1 + s2 + C2))
    return m.mean()


@pytest.mark.parametrize("shape,near", [((1, 3, 37, 53), False), ((2, 3, 70, 90), True),
                                        ((1, 1, 7, 9), False), ((1, 3, 64, 96), True),
                                        ((1, 2, 33, 31), False)])
@pytest.mark.parametrize("padding", ["same", "valid"])
def test_loss_and_gradient_vs_oracle(shape, near, padding):
    if padding == "valid" and min(shape[-2:]) <= 10:
        pytest.skip("'valid' needs images larger than the window")
    img, gt = images(shape, 1, near)
    x = img.to(DEV).requires_grad_(True)
    loss = LS.l1_ssim_loss(x, gt.to(DEV), 0.2, padding=padding)
    loss.backward()
    ms, ml, ol, og = orc.ssim_loss(img.numpy(), gt.numpy(), padding, 0.8, -0.2, 0.2)
    assert abs(loss.item() - ol) < 2e-6, (loss.item(), ol)
    assert rel_max(x.grad.cpu().numpy(), og) < 1e-4
    x2 = img.to(DEV).requires_grad_(True)
    s = LS.ssim(x2, gt.to(DEV), padding=padding)
    (3.0 * s).backward()  # the incoming gradient scales the stored one
    _, _, _, sg = orc.ssim_loss(img.numpy(), gt.numpy(), padding, 0.0, 1.0, 0.0)
    assert abs(s.item() - ms) < 2e-6
    assert rel_max(x2.grad.cpu().numpy(), 3.0 * sg) < 1e-4


def test_channels_last_layout_needs_no_copy():
    """The renderer's [C, H, W, 3] output against [N, 3, H, W]: same loss,
    same gradient (transposed), and a permuted view gives the same again."""
    img, gt = images((2, 45, 67, 3), 2, True)
    a = img.to(DEV).requires_grad_(True)
    la = LS.l1_ssim_loss(a, gt.to(DEV), channels_last=True)
    la.backward()
    b = img.permute(0, 3, 1, 2).contiguous().to(DEV).requires_grad_(True)
    lb = LS.l1_ssim_loss(b, gt.permute(0, 3, 1, 2).contiguous().to(DEV))
    lb.backward()
    assert abs(la.item() - lb.item()) < 1e-6
    assert torch.allclose(a.grad.permute(0, 3, 1, 2), b.grad, rtol=0, atol=1e-9 + 1e-6 * float(
        b.grad.abs().max()))
    c = img.to(DEV).requires_grad_(True)
    lc = LS.l1_ssim_loss(c.permute(0, 3, 1, 2), gt.to(DEV).permute(0, 3, 1, 2))
    lc.backward()
    assert lc.item() == la.item() and torch.equal(c.grad, a.grad)


def test_deterministic():
    img, gt = images((1, 3, 200, 300), 3)
    outs = []
    for _ in range(3):
        x = img.to(DEV).requires_grad_(True)
        l = LS.l1_ssim_loss(x, gt.to(DEV))
        l.backward()
        outs.append((l.item(), x.grad.clone()))
    for l, g in outs[1:]:
        assert l == outs[0][0] and torch.equal(g, outs[0][1])


def test_fused_ssim_dropin_vs_torch_fp32():
    from fused_ssim import fused_ssim
    old = torch.backends.cudnn.allow_tf32
    torch.backends.cudnn.allow_tf32 = False
    try:
        img, gt = images((1, 3, 120, 160), 4, True)
        x = img.to(DEV).requires_grad_(True)
        s = fused_ssim(x, gt.to(DEV))
        s.backward()
        xr = img.to(DEV).requires_grad_(True)
        sr = torch_ssim(xr, gt.to(DEV))
        sr.backward()
        assert abs(s.item() - sr.item()) < 2e-6
        assert rel_max(x.grad.cpu().numpy(), xr.grad.cpu().numpy().astype(np.float64)) < 1e-4
        with torch.no_grad():
            assert abs(fused_ssim(x, gt.to(DEV), train=False).item() - s.item()) < 1e-7
        v = fused_ssim(img.to(DEV), gt.to(DEV), padding="valid")
        assert v.grad_fn is None
    finally:
        torch.backends.cudnn.allow_tf32 = old


def test_full_hd_against_oracle():
    img, gt = images((1, 3, 1080, 1920), 5, True)
    x = img.to(DEV).requires_grad_(True)
    l = LS.l1_ssim_loss(x, gt.to(DEV))
    l.backward()
    _, _, ol, og = orc.ssim_loss(img.numpy(), gt.numpy(), "same", 0.8, -0.2, 0.2)
    assert abs(l.item() - ol) < 2e-6
    assert rel_max(x.grad.cpu().numpy(), og) < 1e-4


def test_captured_in_a_graph():
    img, gt = images((1, 3, 96, 128), 6)
    x = img.to(DEV).requires_grad_(True)
    y = gt.to(DEV)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(2):
            x.grad = None
            LS.l1_ssim_loss(x, y).backward()
    torch.cuda.current_stream().wait_stream(s)
    x.grad = None
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        loss = LS.l1_ssim_loss(x, y)
        loss.backward()
    img2, gt2 = images((1, 3, 96, 128), 7, True)
    with torch.no_grad():
        x.copy_(img2.to(DEV))
        y.copy_(gt2.to(DEV))
    graph.replay()
    graph.replay()  # the ticket counter is back at zero after every launch
    torch.cuda.synchronize()
    _, _, ol, og = orc.ssim_loss(img2.numpy(), gt2.numpy(), "same", 0.8, -0.2, 0.2)
    assert abs(loss.item() - ol) < 2e-6
    assert rel_max(x.grad.cpu().numpy(), og) < 1e-4


def test_errors():
    a = torch.rand(1, 3, 20, 20, device=DEV)
    with pytest.raises(ValueError):
        LS.l1_ssim_loss(a, torch.rand(1, 3, 20, 21, device=DEV))
    with pytest.raises(RuntimeError):
        LS.ssim(torch.rand(1, 3, 8, 30, device=DEV), torch.rand(1, 3, 8, 30, device=DEV),
                padding="valid")
    with pytest.raises(TypeError):
        LS.ssim(a.double(), a.double())
    with pytest.raises(ValueError):
        LS.ssim(a, a, padding="full")


@pytest.mark.parametrize("n", [1, 7, 4096, 6_220_803])
def test_l1_loss_matches_torch(n):
    g = torch.Generator().manual_seed(n)
    x = torch.rand(n, generator=g).to(DEV).requires_grad_(True)
    y = torch.rand(n, generator=g).to(DEV)
    y[: n // 3] = x.detach()[: n // 3]  # ties: the gradient is 0 there, as torch's sign
    l = LS.l1_loss(x, y)
    (2.0 * l).backward()
    xr = x.detach().clone().requires_grad_(True)
    lr = (xr - y).abs().mean()
    (2.0 * lr).backward()
    assert abs(l.item() - lr.item()) <= 1e-6 * abs(lr.item())
    assert torch.equal(x.grad, xr.grad)
