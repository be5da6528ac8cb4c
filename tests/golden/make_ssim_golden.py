"""Golden vectors for the training loss from the reference's own SSIM.

The reference defines SSIM in plain PyTorch (utils/loss_utils.py:26-80); its
training loop evaluates the same function through the fused_ssim package
(train.py:117-121, not installed here).  This script imports loss_utils from a
checkout of the reference, evaluates ssim() and the training loss
0.8 L1 + 0.2 (1 - ssim) on small seeded images on the CPU, in float32 and in
float64 (the reference builds its window in float32 either way), takes the
autograd gradients (stored as float32) w.r.t. the rendered image, and stores everything in
ssim.npz next to this script.

Usage:  python tests/golden/make_ssim_golden.py /path/to/reference
"""
import importlib.util
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("UBS_REFERENCE_ROOT")
if not REF:
    sys.exit("usage: %s /path/to/reference (or set UBS_REFERENCE_ROOT)" % sys.argv[0])
spec = importlib.util.spec_from_file_location("ref_loss_utils",
                                              os.path.join(REF, "utils", "loss_utils.py"))
lu = importlib.util.module_from_spec(spec)
spec.loader.exec_module(lu)

LAMBDA_DSSIM = 0.2  # arguments/__init__.py default


def case(g, shape, near=False):
    gt = torch.rand(*shape, generator=g)
    if near:  # a rendering close to its target, as late in training
        img = (gt + 0.05 * torch.randn(*shape, generator=g)).clamp(0, 1)
    else:
        img = torch.rand(*shape, generator=g)
    return img, gt


def evaluate(img, gt, dtype):
    x = img.to(dtype).requires_grad_(True)
    y = gt.to(dtype)
    s = lu.ssim(x, y)
    (gs,) = torch.autograd.grad(s, x)
    x2 = img.to(dtype).requires_grad_(True)
    loss = (1.0 - LAMBDA_DSSIM) * lu.l1_loss(x2, y) + LAMBDA_DSSIM * (1.0 - lu.ssim(x2, y))
    (gl,) = torch.autograd.grad(loss, x2)
    return s.item(), gs.numpy(), loss.item(), gl.numpy()


def main():
    g = torch.Generator().manual_seed(0)
    shapes = [((1, 3, 37, 53), False), ((2, 3, 20, 31), False), ((1, 1, 7, 9), False),
              ((1, 3, 40, 40), True)]
    out = {}
    for i, (shape, near) in enumerate(shapes):
        img, gt = case(g, shape, near)
        out["img%d" % i] = img.numpy()
        out["gt%d" % i] = gt.numpy()
        for tag, dt in (("f32", torch.float32), ("f64", torch.float64)):
            s, gs, loss, gl = evaluate(img, gt, dt)
            out["ssim%d_%s" % (i, tag)] = np.float64(s)
            out["ssim_grad%d_%s" % (i, tag)] = gs.astype(np.float32)
            out["loss%d_%s" % (i, tag)] = np.float64(loss)
            out["loss_grad%d_%s" % (i, tag)] = gl.astype(np.float32)
    out["n_cases"] = np.int32(len(shapes))
    out["lambda_dssim"] = np.float64(LAMBDA_DSSIM)
    np.savez_compressed(os.path.join(HERE, "ssim.npz"), **out)
    print("wrote ssim.npz", len(shapes), "cases")


if __name__ == "__main__":
    main()
