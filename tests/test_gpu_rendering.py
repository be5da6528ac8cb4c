"""gsplat.rendering.rasterization() (the reference's pipeline entry point,
rendering.py:17-232) in every render mode the reference handles, against the
oracle's projection, intersections and blend of the channels that mode
builds: RGB, Depth, EDepth, RGB+D, RGB+ED (expected-depth normalisation,
which the reference applies only to "RGB+ED" since it tests for "ED"),
Normal, antialiased compensation, backgrounds with the appended depth
channel, and channel chunking above 32 channels."""
import numpy as np
import pytest
import torch

import oracle as orc
from gsplat.rendering import rasterization
from gsplat.utils import depth_to_normal
from ubs import scene as S

pytestmark = pytest.mark.gpu
DEV = "cuda"
W, H, TS = 160, 120, 16


def scene(N=3000, seed=0, channels=3):
    g = torch.Generator().manual_seed(seed)
    means = (torch.rand(N, 3, generator=g) * 2 - 1) * 1.0
    A = torch.randn(N, 3, 3, generator=g) * 0.06
    covars = A @ A.transpose(1, 2) + torch.eye(3) * 1e-3
    opac = torch.rand(N, generator=g) * 0.8 + 0.1
    betas = torch.rand(N, generator=g) * 2 + 0.3
    colors = torch.rand(N, channels, generator=g)
    cam = S.orbit_view(seed + 3, 3.0, W, H, 150.0, 150.0)
    return means, covars, opac, betas, colors, cam


def ours(means, covars, opac, betas, colors, cam, mode, bg=None, aa=False):
    rc, ra, meta = rasterization(
        means.to(DEV), None, None, opac.to(DEV), betas.to(DEV), colors.to(DEV),
        cam.viewmat[None].to(DEV), cam.K[None].to(DEV), W, H, tile_size=TS,
        backgrounds=None if bg is None else bg.to(DEV), render_mode=mode,
        rasterize_mode="antialiased" if aa else "classic", covars=covars.to(DEV))
    return rc[0].cpu().numpy(), ra[0].cpu().numpy(), meta


def oracle(meta, colors_fn, bg=None):
    """The oracle's FP64 blend of the colours a mode builds (colors_fn(depths
    [N]) -> [N, D]) over the projection and sorted intersections in `meta`;
    the projection and the sort have their own parity tests.  (The FP32
    oracle's own rounding is of the order of the 1e-5 tolerance.)"""
    npy = lambda t: t.detach().cpu().numpy()  # noqa: E731
    d = npy(meta["depths"])
    cols = colors_fn(d[0])[None]
    oc, oa, _ = orc.rasterize_to_pixels(npy(meta["means2d"]), npy(meta["conics"]), cols,
                                        npy(meta["opacities"]), npy(meta["betas"]), W, H, TS,
                                        npy(meta["isect_offsets"]), npy(meta["flatten_ids"]),
                                        backgrounds=None if bg is None else bg[None],
                                        dtype=np.float64)
    return oc[0], oa[0]


def oracle_compensation(means, covars, cam):
    c6 = covars[:, [0, 0, 0, 1, 1, 2], [0, 1, 2, 1, 2, 2]].numpy()
    vm, K = cam.viewmat.numpy()[None], cam.K.numpy()[None]
    radii, _, _, _, comp = orc.fully_fused_projection(means.numpy(), c6, None, None, vm, K, W, H,
                                                      calc_compensations=True)
    return comp[0], radii[0]


def close(a, b, tol=1e-5):
    assert a.shape == b.shape, (a.shape, b.shape)
    err = np.abs(a - b) / np.maximum(1.0, np.abs(b))
    assert float(err.max()) < tol, float(err.max())


@pytest.mark.parametrize("aa", [False, True])
def test_rgb_and_antialiased(aa):
    m, c, o, b, col, cam = scene(seed=1)
    bg = np.array([0.2, 0.3, 0.1], np.float32)
    rc, ra, meta = ours(m, c, o, b, col, cam, "RGB", torch.from_numpy(bg[None]), aa)
    oc, oa = oracle(meta, lambda d: col.numpy(), bg)
    close(rc, oc)
    close(ra, oa)
    if aa:  # opacities carry the antialiasing compensation
        comp, radii = oracle_compensation(m, c, cam)
        vis = radii > 0
        got = meta["opacities"][0].cpu().numpy()
        assert np.allclose(got[vis], o.numpy()[vis] * comp[vis], rtol=1e-5, atol=1e-7)
    for key in ("camera_ids", "primitive_ids", "radii", "means2d", "depths", "conics",
                "opacities", "betas", "tile_width", "tile_height", "tiles_per_gauss",
                "isect_ids", "flatten_ids", "isect_offsets", "width", "height", "tile_size",
                "n_cameras"):
        assert key in meta, key


@pytest.mark.parametrize("mode", ["RGB+D", "RGB+ED"])
def test_rgb_plus_depth_modes(mode):
    m, c, o, b, col, cam = scene(seed=2)
    bg = np.array([0.2, 0.3, 0.1], np.float32)
    rc, ra, meta = ours(m, c, o, b, col, cam, mode, torch.from_numpy(bg[None]))
    oc, oa = oracle(meta, lambda d: np.concatenate([col.numpy(), d[:, None]], 1),
                    np.concatenate([bg, [0.0]]).astype(np.float32))
    assert rc.shape == (H, W, 4)
    close(rc[..., :3], oc[..., :3])
    depth = rc[..., 3:]
    if mode == "RGB+ED":
        # expected depth = accumulated depth / max(alpha, 1e-10); undone here,
        # since the division amplifies rounding wherever alpha is tiny
        depth = depth * np.maximum(ra, 1e-10)
    # depth (values ~3-4): FP32 accumulation error grows with the channel's
    # magnitude over hundreds of contributions
    close(depth, oc[..., 3:], 3e-5)
    close(ra, oa)


@pytest.mark.parametrize("mode", ["Depth", "EDepth"])
def test_depth_modes(mode):
    m, c, o, b, col, cam = scene(seed=3)
    rc, ra, meta = ours(m, c, o, b, col, cam, mode, torch.tensor([[0.5, 0.5, 0.5]]))
    # the reference replaces the background with zeros and, testing for "ED",
    # leaves "EDepth" unnormalised
    oc, oa = oracle(meta, lambda d: d[:, None], np.zeros(1, np.float32))
    assert rc.shape == (H, W, 1)
    close(rc, oc)
    close(ra, oa)


def test_normal_mode():
    """Normal = (normals of the rendered depth + 1) / 2, world frame."""
    m, c, o, b, col, cam = scene(seed=4)
    rc, _, _ = ours(m, c, o, b, col, cam, "Normal")
    depth, _, _ = ours(m, c, o, b, col, cam, "Depth")
    c2w = torch.inverse(cam.viewmat.to(DEV))[None]
    expect = (depth_to_normal(torch.from_numpy(depth).to(DEV)[None], c2w,
                              cam.K[None].to(DEV))[0] + 1) / 2
    assert rc.shape == (H, W, 3)
    close(rc, expect.cpu().numpy(), 1e-6)


def test_channel_chunks_above_32():
    m, c, o, b, col, cam = scene(seed=5, channels=40)
    rc, ra, meta = ours(m, c, o, b, col, cam, "RGB")
    oc, oa = oracle(meta, lambda d: col.numpy())
    assert rc.shape == (H, W, 40)
    close(rc, oc)
    close(ra, oa)


def test_depth_to_normal_definition():
    """Normals from central differences of the back-projected depth map."""
    cam = S.orbit_view(9, 3.0, 32, 24, 30.0, 30.0)
    g = torch.Generator().manual_seed(0)
    depth = 2.0 + 0.1 * torch.rand(1, 24, 32, 1, generator=g)
    c2w = torch.inverse(cam.viewmat)[None]
    n = depth_to_normal(depth, c2w, cam.K[None])[0].numpy()
    K = cam.K.numpy()
    ys, xs = np.meshgrid(np.arange(24) + 0.5, np.arange(32) + 0.5, indexing="ij")
    cam_pts = np.stack([(xs - K[0, 2]) / K[0, 0], (ys - K[1, 2]) / K[1, 1], np.ones_like(xs)],
                       -1) * depth[0].numpy()
    world = cam_pts @ c2w[0, :3, :3].numpy().T + c2w[0, :3, 3].numpy()
    d_rows = world[2:, 1:-1] - world[:-2, 1:-1]  # along the image's rows (y)
    d_cols = world[1:-1, 2:] - world[1:-1, :-2]  # along its columns (x)
    nn = np.cross(d_rows, d_cols)
    nn /= np.linalg.norm(nn, axis=-1, keepdims=True)
    assert np.allclose(n[1:-1, 1:-1], nn, atol=1e-4)
    assert not n[0].any() and not n[-1].any() and not n[:, 0].any() and not n[:, -1].any()


def test_empty_scene_renders_background():
    """rasterization() of no primitives: the background, zero alpha, as the
    reference (its kernels see empty ranges everywhere)."""
    cam = S.orbit_view(1, 3.0, W, H, 150.0, 150.0)
    bg = torch.tensor([[0.2, 0.4, 0.6]], device=DEV)
    e3 = torch.zeros(0, 3, device=DEV)
    rc, ra, meta = rasterization(e3, None, None, torch.zeros(0, device=DEV),
                                 torch.zeros(0, device=DEV), e3, cam.viewmat[None].to(DEV),
                                 cam.K[None].to(DEV), W, H, tile_size=TS, backgrounds=bg,
                                 covars=torch.zeros(0, 3, 3, device=DEV))
    assert torch.equal(rc[0], bg[0].expand(H, W, 3)) and not ra.any()
    assert meta["flatten_ids"].numel() == 0
