"""The reference's training loss in two kernel launches (csrc/ssim.cu).

train.py:117-121 trains on  (1 - l) L1(image, gt) + l (1 - SSIM(image, gt))
(l = lambda_dssim, 0.2) with SSIM from the fused_ssim package, which
evaluates utils/loss_utils.py:26-80's definition.  `l1_ssim_loss` computes
that loss and writes d loss / d image in the same launches (the backward
pass only scales it by the incoming gradient); `ssim` is the SSIM term
alone and `l1_loss` the L1 term alone (utils/loss_utils.py:18-19), one
launch with its gradient.

Images may be laid out as [..., C, H, W] or, with channels_last=True, as
[..., H, W, C] (the renderer's layout) with any strides: nothing is copied.
"""
import torch

from . import _lib as L

_W_SSIM_ONLY = (0.0, 1.0, 0.0)


def _dims(t, channels_last):
    """(n, c, h, w) sizes and element strides of t viewed as images."""
    if t.dim() not in (3, 4):
        raise ValueError("expected [C, H, W] / [N, C, H, W] images (or the channels-last "
                         "forms), got %s" % (tuple(t.shape),))
    if channels_last:
        h, w, c = t.shape[-3:]
        sh, sw, sc = t.stride()[-3:]
    else:
        c, h, w = t.shape[-3:]
        sc, sh, sw = t.stride()[-3:]
    n = t.shape[0] if t.dim() == 4 else 1
    sn = t.stride(0) if t.dim() == 4 else 0
    return (n, c, h, w), (sn, sc, sh, sw)


def _check(img, gt, channels_last):
    if not (img.is_cuda and gt.is_cuda):
        raise TypeError("the loss kernel needs CUDA tensors")
    if img.dtype != torch.float32 or gt.dtype != torch.float32:
        raise TypeError("the loss kernel handles float32 images")
    if img.shape != gt.shape:
        raise ValueError("image and target shapes differ: %s vs %s"
                         % (tuple(img.shape), tuple(gt.shape)))
    return _dims(img, channels_last)


def _launch(img, gt, grad, channels_last, valid, weights):
    import ctypes
    (n, c, h, w), si = _dims(img, channels_last)
    _, sg = _dims(gt, channels_last)
    sd = _dims(grad, channels_last)[1] if grad is not None else None
    dev = img.device
    out = torch.empty(3, dtype=torch.float32, device=dev)
    # the ticket counter (first bytes) must start at zero; the rest is written
    # before it is read
    ws = torch.empty(int(L.query("ubs_ssim_workspace_bytes", n, c, h, w)), dtype=torch.uint8,
                     device=dev)
    ws[:256].zero_()
    arr = lambda s: (ctypes.c_int64 * 4)(*s)  # noqa: E731
    si_c, sg_c = arr(si), arr(sg)
    sd_c = arr(sd) if sd is not None else None
    L.call("ubs_ssim_loss", L.strided_ptr(img), ctypes.cast(si_c, ctypes.c_void_p),
           L.strided_ptr(gt), ctypes.cast(sg_c, ctypes.c_void_p),
           L.strided_ptr(grad) if grad is not None else None,
           ctypes.cast(sd_c, ctypes.c_void_p) if sd_c is not None else None, n, c, h, w,
           1 if valid else 0, float(weights[0]), float(weights[1]), float(weights[2]),
           L.ptr(out), L.ptr(ws), ws.numel(), L.stream(dev))
    return out


class _Loss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, img, gt, channels_last, valid, weights, index):
        grad = None
        if ctx.needs_input_grad[0]:
            grad = torch.empty_like(img)
        out = _launch(img.detach(), gt.detach(), grad, channels_last, valid, weights)
        ctx.save_for_backward(grad)
        return out[index]

    @staticmethod
    def backward(ctx, g):
        (grad,) = ctx.saved_tensors
        return grad * g, None, None, None, None, None


def _apply(img, gt, channels_last, valid, weights, index):
    _check(img, gt, channels_last)
    if torch.is_grad_enabled() and img.requires_grad:
        return _Loss.apply(img, gt.detach(), channels_last, valid, weights, index)
    with torch.no_grad():
        return _launch(img.detach(), gt.detach(), None, channels_last, valid, weights)[index]


def l1_ssim_loss(img, gt, lambda_dssim=0.2, channels_last=False, padding="same"):
    """(1 - lambda_dssim) mean|img - gt| + lambda_dssim (1 - SSIM(img, gt)),
    train.py:117-121's loss, as a 0-dim tensor differentiable w.r.t. img."""
    if padding not in ("same", "valid"):
        raise ValueError("padding must be 'same' or 'valid'")
    lam = float(lambda_dssim)
    return _apply(img, gt, channels_last, padding == "valid", (1.0 - lam, -lam, lam), 2)


def ssim(img, gt, channels_last=False, padding="same"):
    """Mean SSIM of img against gt (utils/loss_utils.py:45-80 with size_average),
    differentiable w.r.t. img."""
    if padding not in ("same", "valid"):
        raise ValueError("padding must be 'same' or 'valid'")
    return _apply(img, gt, channels_last, padding == "valid", _W_SSIM_ONLY, 0)


class _L1(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, y):
        grad = torch.empty_like(x) if ctx.needs_input_grad[0] else None
        out = _l1_launch(x.detach(), y.detach(), grad)
        ctx.save_for_backward(grad)
        return out[0]

    @staticmethod
    def backward(ctx, g):
        (grad,) = ctx.saved_tensors
        return grad * g, None


def _l1_launch(x, y, grad):
    n = x.numel()
    dev = x.device
    out = torch.empty(2, dtype=torch.float32, device=dev)
    ws = torch.empty(int(L.query("ubs_l1_loss_workspace_bytes", n)), dtype=torch.uint8,
                     device=dev)
    ws[:256].zero_()
    L.call("ubs_l1_loss", L.ptr(x), L.ptr(y), L.ptr(grad) if grad is not None else None, n,
           1.0, L.ptr(out), L.ptr(ws), ws.numel(), L.stream(dev))
    return out


def l1_loss(img, gt):
    """mean |img - gt| (utils/loss_utils.py:18-19) of two contiguous float32
    CUDA tensors of one shape, differentiable w.r.t. img; one launch writes
    the value and the gradient."""
    if not (img.is_cuda and gt.is_cuda) or img.dtype != torch.float32 or \
            gt.dtype != torch.float32:
        raise TypeError("l1_loss needs float32 CUDA tensors")
    if img.shape != gt.shape:
        raise ValueError("shapes differ: %s vs %s" % (tuple(img.shape), tuple(gt.shape)))
    if not (img.is_contiguous() and gt.is_contiguous()):
        raise ValueError("l1_loss needs contiguous tensors")
    if torch.is_grad_enabled() and img.requires_grad:
        return _L1.apply(img, gt.detach())
    with torch.no_grad():
        return _l1_launch(img.detach(), gt.detach(), None)[0]
