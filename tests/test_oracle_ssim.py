"""Pin the oracle's training loss (FP64 SSIM + L1 and the analytic gradient)
against the reference's own PyTorch SSIM (tests/golden/make_ssim_golden.py
ran utils/loss_utils.py) and against finite differences.  CPU only."""
import os

import numpy as np
import pytest

import oracle as orc

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ssim.npz")


def rel_max(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).max() / np.abs(b).max())


@pytest.mark.parametrize("tag,tol_v,tol_g", [("f64", 1e-6, 2e-6), ("f32", 1e-6, 1e-5)])
def test_oracle_matches_reference_ssim(tag, tol_v, tol_g):
    """The reference rounds its window to float32 even in float64, which
    alone moves the map by ~2e-7; float32 adds its own rounding."""
    z = np.load(GOLD)
    lam = float(z["lambda_dssim"])
    for i in range(int(z["n_cases"])):
        x, y = z["img%d" % i], z["gt%d" % i]
        ms, _, _, grad = orc.ssim_loss(x, y, "same", 0.0, 1.0, 0.0)
        assert abs(ms - float(z["ssim%d_%s" % (i, tag)])) < tol_v
        assert rel_max(grad, z["ssim_grad%d_%s" % (i, tag)]) < tol_g
        _, _, loss, lgrad = orc.ssim_loss(x, y, "same", 1 - lam, -lam, lam)
        assert abs(loss - float(z["loss%d_%s" % (i, tag)])) < tol_v
        assert rel_max(lgrad, z["loss_grad%d_%s" % (i, tag)]) < tol_g


@pytest.mark.parametrize("padding", ["same", "valid"])
def test_oracle_gradient_finite_differences(padding):
    rng = np.random.default_rng(1)
    x, y = rng.random((2, 2, 14, 17)), rng.random((2, 2, 14, 17))
    w = (0.8, -0.2, 0.2)
    _, _, _, grad = orc.ssim_loss(x, y, padding, *w)
    eps = 1e-6
    for idx in [(0, 0, 0, 0), (1, 1, 7, 8), (0, 1, 13, 16), (1, 0, 5, 5), (0, 0, 2, 12)]:
        xp, xm = x.copy(), x.copy()
        xp[idx] += eps
        xm[idx] -= eps
        fd = (orc.ssim_loss(xp, y, padding, *w)[2] - orc.ssim_loss(xm, y, padding, *w)[2]) / (2 * eps)
        assert abs(fd - grad[idx]) <= 1e-7 + 1e-5 * abs(fd), (idx, fd, grad[idx])


def test_oracle_valid_padding_crops_the_map():
    rng = np.random.default_rng(2)
    x, y = rng.random((1, 1, 20, 24)), rng.random((1, 1, 20, 24))
    ms_valid = orc.ssim_loss(x, y, "valid")[0]
    # the same mean from the full map of a crop-free definition
    g = orc.ssim_window()
    blur = lambda a: orc._blur(a, g)  # noqa: E731
    mx, my = blur(x), blur(y)
    vx, vy, cxy = blur(x * x) - mx ** 2, blur(y * y) - my ** 2, blur(x * y) - mx * my
    smap = ((2 * mx * my + orc.SSIM_C1) * (2 * cxy + orc.SSIM_C2) /
            ((mx ** 2 + my ** 2 + orc.SSIM_C1) * (vx + vy + orc.SSIM_C2)))
    assert abs(ms_valid - smap[..., 5:-5, 5:-5].mean()) < 1e-14
