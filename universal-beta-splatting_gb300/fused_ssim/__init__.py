"""Drop-in for the fused_ssim package the reference trains and evaluates with
(train.py:17,120; scene/__init__.py:26,191; pinned in setup.py:26).

fused_ssim(img1, img2, padding="same", train=True) returns the mean SSIM of
img1 [N, C, H, W] against img2 as a 0-dim tensor, differentiable w.r.t. img1
(img2 is the target), with SSIM as utils/loss_utils.py:26-80 defines it.  The
whole computation, gradient included, is one call of the library's loss
(ubs.loss: a statistics kernel and a gradient kernel); train=False skips the
gradient kernel.
"""
import torch

from ubs import loss as _loss

__all__ = ["fused_ssim"]


def fused_ssim(img1, img2, padding="same", train=True):
    if padding not in ("same", "valid"):
        raise ValueError("padding must be 'same' or 'valid'")
    if img1.dim() != 4:
        raise ValueError("fused_ssim expects [N, C, H, W] images")
    if not train:
        with torch.no_grad():
            return _loss.ssim(img1, img2, padding=padding)
    return _loss.ssim(img1, img2, padding=padding)
