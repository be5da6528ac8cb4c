"""Gradients of the batched 7-D (dynamic) render on a 2,000-primitive 64x64
subset of the 500k / 8-view configuration:

* against the reference's own CUDA kernels (oracle/ref_gpu.py, one view per
  launch): images within 1e-5 max abs, every parameter's gradient within 1e-4
  relative (L2), with the reference's conditioning backward;
* against FP64 central finite differences of the oracle's full render chain
  (activations, rotation, covariance, conditioning, projection,
  intersections, blend), with the exact conditioning backward: per
  coordinate |g - fd| <= 2e-3 |fd| + 1e-4 max|fd|.  The view-direction query
  is held at its unperturbed value, because the reference's conditioning
  operator passes no gradient to its query (_wrapper.py:611 returns None for
  it), so xyz receives no gradient through normalize(xyz - camera_center).
"""
import numpy as np
import pytest
import torch

import oracle as orc
from ubs import scene as S
from ubs.render import Renderer, Views

pytestmark = pytest.mark.gpu
DEV = "cuda"
W = H = 64
TS = 16
F = 1056.25 * 64 / 1352  # the configuration's field of view at 64 pixels


def subset(seed=0, n=2000):
    p = S.synthetic_params(n, 7, seed=seed, xyz_range=1.0, device="cpu")
    p["scale"][:, :3] += 2.0  # footprints of a few pixels at 64x64
    return p


def cameras():
    return [S.orbit_view(10 + i, 3.0, W, H, F, F, timestamp=t, device=DEV)
            for i, t in enumerate((0.15, 0.6, 0.85))]


def fused(p, cams, weights, exact):
    leaves = {k: v.to(DEV).clone().requires_grad_(True) for k, v in p.items()}
    r = Renderer(dim=7, exact_cond_grad=exact)
    views = Views(cams, device=DEV)
    colors, _ = r.render(leaves, views, torch.zeros(len(cams), 3, device=DEV))
    imgs = views.split(colors)
    loss = sum((im * w).sum() for im, w in zip(imgs, weights))
    loss.backward()
    return [im.detach() for im in imgs], {k: v.grad.detach().cpu().double() for k, v in leaves.items()}


def test_7d_batched_matches_reference_kernels():
    ref_gpu = pytest.importorskip("ref_gpu")
    if not ref_gpu.available():
        pytest.skip("reference kernels not built")
    rp = ref_gpu.RefPipeline()
    p = subset(1)
    cams = cameras()
    g = torch.Generator().manual_seed(2)
    weights = [torch.randn(H, W, 3, generator=g).to(DEV) for _ in cams]
    imgs, grads = fused(p, cams, weights, exact=False)
    leaves = {k: v.to(DEV).clone().requires_grad_(True) for k, v in p.items()}
    ri, rj = S.rest_indices(7, DEV)
    total = 0.0
    for c, w, im in zip(cams, weights, imgs):
        img_r, _, _ = rp.render_view(leaves, c.viewmat, c.K, W, H, c.center,
                                     torch.zeros(3, device=DEV), ri, rj, tile_size=TS,
                                     timestamp=c.timestamp)
        img_r = img_r.permute(1, 2, 0)
        assert float((im - img_r.detach()).abs().max()) < 1e-5
        total = total + (img_r * w).sum()
    total.backward()
    for k in grads:
        ref = leaves[k].grad.detach().cpu().double()
        rel = float((grads[k] - ref).norm() / ref.norm().clamp_min(1e-30))
        assert rel < 1e-4, (k, rel)


def oracle_queries(p, cams):
    out = []
    for c in cams:
        vm = c.viewmat.double().cpu().numpy()
        center = -vm[:3, :3].T @ vm[:3, 3]
        vd = p["xyz"] - center[None]
        q = vd / np.linalg.norm(vd, axis=-1, keepdims=True)
        out.append(np.concatenate([q, np.full((len(q), 1), c.timestamp)], 1))
    return out


def oracle_loss64(p, cams, weights, queries=None):
    """FP64 render of every view through the oracle; sum of weighted images.
    `queries` fixes the conditioning queries (default: from p)."""
    f64 = np.float64
    sp = np.log1p(np.exp(-np.abs(p["scale"]))) + np.maximum(p["scale"], 0)
    beta = 4.0 * np.exp(p["beta"])
    opac = 1.0 / (1.0 + np.exp(-p["opacity"]))
    ri, rj = (t.numpy() for t in S.rest_indices(7))
    R = orc.l_triangle_to_rotmat(p["l_triangle"], dtype=f64)
    cov = orc.rot_scale_l_triangle_to_covar(R, sp, p["l_triangle"], ri, rj, dtype=f64)
    m_nd = np.concatenate([p["xyz"], p["mean"]], 1)
    iu = ([0, 0, 0, 1, 1, 2], [0, 1, 2, 1, 2, 2])
    tw, th = (W + TS - 1) // TS, (H + TS - 1) // TS
    total = 0.0
    if queries is None:
        queries = oracle_queries(p, cams)
    for c, w, q in zip(cams, weights, queries):
        vm = c.viewmat.double().cpu().numpy()
        K = c.K.double().cpu().numpy()
        om, oV, oo = orc.cond_mean_convariance_opacity(m_nd, cov, opac, beta[:, 1:], q, dtype=f64)
        c6 = np.ascontiguousarray(oV[:, iu[0], iu[1]])
        radii, m2, d, cn, _ = orc.fully_fused_projection(om, c6, None, None, vm[None], K[None],
                                                         W, H, dtype=f64)
        _, ids, fl = orc.isect_tiles(m2, radii, d, TS, tw, th)
        offs = orc.isect_offset_encode(ids, 1, tw, th)
        oc, _, _ = orc.rasterize_to_pixels(m2, cn, p["rgb"][None], oo.reshape(1, -1),
                                           beta[:, 0].reshape(1, -1), W, H, TS, offs, fl,
                                           backgrounds=np.zeros((1, 3)), dtype=f64)
        total += float((oc[0] * w).sum())
    return total


def test_7d_exact_gradients_vs_fp64_finite_differences():
    p = subset(3)
    cams = cameras()
    g = torch.Generator().manual_seed(4)
    weights = [torch.randn(H, W, 3, generator=g) for _ in cams]
    _, grads = fused(p, cams, [w.to(DEV) for w in weights], exact=True)
    p64 = {k: v.double().numpy().copy() for k, v in p.items()}
    w64 = [w.double().numpy() for w in weights]
    # the primitives with the largest spatial gradients, one coordinate per
    # parameter group each
    order = torch.argsort(-grads["xyz"].norm(dim=1))[:4].tolist()
    coords = []
    for n in order:
        for k in ("xyz", "mean", "scale", "l_triangle", "opacity", "beta", "rgb"):
            j = int(torch.argmax(grads[k][n].abs()))
            coords.append((k, n, j))
    h = 1e-6
    q0 = oracle_queries(p64, cams)
    fd, an = [], []
    for k, n, j in coords:
        x0 = p64[k][n, j]
        p64[k][n, j] = x0 + h
        lp = oracle_loss64(p64, cams, w64, q0)
        p64[k][n, j] = x0 - h
        lm = oracle_loss64(p64, cams, w64, q0)
        p64[k][n, j] = x0
        fd.append((lp - lm) / (2 * h))
        an.append(float(grads[k][n, j]))
    fd, an = np.array(fd), np.array(an)
    tol = 2e-3 * np.abs(fd) + 1e-4 * np.abs(fd).max()
    bad = [(coords[i], an[i], fd[i]) for i in range(len(fd)) if abs(an[i] - fd[i]) > tol[i]]
    assert not bad, bad
