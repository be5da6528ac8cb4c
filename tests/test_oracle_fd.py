"""FP64 central finite-difference checks of the oracle's backward passes
(blend and projection), on small scenes away from the non-smooth regimes
(sigma = 1 edge, 0.999 clamp, T <= 1e-4 termination).  CPU only."""
import numpy as np
import pytest

import oracle as orc

F64 = np.float64


def blend_scene(seed, N=24, W=40, H=36, cdim=3):
    rng = np.random.default_rng(seed)
    means2d = np.stack([rng.uniform(4, W - 4, N), rng.uniform(4, H - 4, N)], -1)[None]
    # well-conditioned conics: ellipses of 6..14 px semi-axes
    a = rng.uniform(6, 14, N)
    b = rng.uniform(6, 14, N)
    th = rng.uniform(0, np.pi, N)
    c, s = np.cos(th), np.sin(th)
    cov = np.stack([a * a * c * c + b * b * s * s, (a * a - b * b) * c * s,
                    a * a * s * s + b * b * c * c], -1)
    det = cov[:, 0] * cov[:, 2] - cov[:, 1] ** 2
    conics = np.stack([cov[:, 2] / det, -cov[:, 1] / det, cov[:, 0] / det], -1)[None]
    colors = rng.uniform(0, 1, (1, N, cdim))
    opac = rng.uniform(0.05, 0.5, (1, N))
    betas = rng.uniform(0.5, 3.0, (1, N))
    depths = rng.uniform(1, 5, (1, N)).astype(np.float32)
    radii = np.ceil(np.maximum(a, b)).astype(np.int32)[None] + 1
    return means2d, conics, colors, opac, betas, depths, radii


def render(means2d, conics, colors, opac, betas, W, H, offs, fl, bg):
    return orc.rasterize_to_pixels(means2d, conics, colors, opac, betas, W, H, 16, offs, fl,
                                   backgrounds=bg, dtype=F64)


@pytest.mark.parametrize("with_bg", [False, True])
def test_blend_bwd_matches_central_differences(with_bg):
    W, H = 40, 36
    m2, cn, col, op, be, dp, radii = blend_scene(1)
    tw, th = (W + 15) // 16, (H + 15) // 16
    _, ids, fl = orc.isect_tiles(m2.astype(np.float32), radii, dp, 16, tw, th)
    offs = orc.isect_offset_encode(ids, 1, tw, th)
    bg = np.array([[0.2, 0.5, 0.9]]) if with_bg else None
    rng = np.random.default_rng(7)
    wc = rng.normal(size=(1, H, W, 3))
    wa = rng.normal(size=(1, H, W, 1))

    def loss(m2_, cn_, col_, op_, be_):
        oc, oa, _ = render(m2_, cn_, col_, op_, be_, W, H, offs, fl, bg)
        return (oc * wc).sum() + (oa * wa).sum()

    oc, oa, li = render(m2, cn, col, op, be, W, H, offs, fl, bg)
    vm2, vcn, vcol, vo, vb = orc.rasterize_to_pixels_bwd(
        m2, cn, col, op, be, W, H, 16, offs, fl, oa, li, wc, wa, backgrounds=bg, dtype=F64)
    params = [m2, cn, col, op, be]
    grads = [vm2, vcn, vcol, vo, vb]
    eps = 1e-6
    for pi in range(5):
        flat = params[pi].reshape(-1)
        for k in rng.choice(flat.size, size=min(12, flat.size), replace=False):
            orig = flat[k]
            flat[k] = orig + eps
            lp = loss(*params)
            flat[k] = orig - eps
            lm = loss(*params)
            flat[k] = orig
            fd = (lp - lm) / (2 * eps)
            an = grads[pi].reshape(-1)[k]
            assert abs(fd - an) <= 1e-5 + 1e-4 * abs(fd), (pi, k, fd, an)


def test_projection_bwd_matches_central_differences():
    rng = np.random.default_rng(3)
    N = 40
    means = rng.uniform(-0.5, 0.5, (N, 3))
    L = rng.normal(size=(N, 3, 3)) * 0.05
    cov = L @ L.transpose(0, 2, 1) + 1e-3 * np.eye(3)
    c6 = np.ascontiguousarray(cov[:, [0, 0, 0, 1, 1, 2], [0, 1, 2, 1, 2, 2]])
    vm = np.eye(4)[None].copy()
    vm[0, 2, 3] = 4.0
    K = np.array([[[120.0, 0, 64], [0, 120.0, 48], [0, 0, 1]]])
    W, H = 128, 96
    radii, m2, d, cn, _ = orc.fully_fused_projection(means, c6, None, None, vm, K, W, H, dtype=F64)
    assert (radii > 0).all()
    wm = rng.normal(size=m2.shape)
    wd = rng.normal(size=d.shape)
    wc = rng.normal(size=cn.shape)

    def loss(means_, c6_):
        _, m2_, d_, cn_, _ = orc.fully_fused_projection(means_, c6_, None, None, vm, K, W, H,
                                                        dtype=F64)
        return (m2_ * wm).sum() + (d_ * wd).sum() + (cn_ * wc).sum()

    gm, gc, _, _, _ = orc.fully_fused_projection_bwd(means, c6, None, None, vm, K, W, H, 0.3,
                                                     radii, cn, None, wm, wd, wc, dtype=F64)
    eps = 1e-6
    for arr, g in ((means, gm), (c6, gc)):
        flat = arr.reshape(-1)
        for k in range(0, flat.size, 7):
            o = flat[k]
            flat[k] = o + eps
            lp = loss(means, c6)
            flat[k] = o - eps
            lm = loss(means, c6)
            flat[k] = o
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - g.reshape(-1)[k]) <= 1e-5 + 1e-4 * abs(fd), (k, fd, g.reshape(-1)[k])
