"""Every occupancy variant of the blend kernels (ubs_set_blend_variant) renders
the same images, and its gradients agree up to the order of the backward's
atomic sums; the autotuner picks a configuration on the GPU and leaves it
set."""
import pytest
import torch

from ubs import scene as S
from ubs.autotune import TileAutotuner, get_blend_variant, set_blend_variant
from ubs.render import Renderer, Views

pytestmark = pytest.mark.gpu
DEV = "cuda"


def scene():
    p = S.synthetic_params(20000, 6, seed=3, xyz_range=1.0, device=DEV)
    p["scale"][:, :3] += 1.0
    cams = [S.orbit_view(5, 3.0, 640, 480, 500.0, 500.0, device=DEV)]
    return p, cams


def render(p, cams, ts, w):
    leaves = {k: v.clone().requires_grad_(True) for k, v in p.items()}
    colors, alphas = Renderer(dim=6, tile_size=ts).render(leaves, Views(cams, tile_size=ts,
                                                                          device=DEV))
    ((colors * w).sum() + alphas.sum()).backward()
    return colors.detach(), {k: v.grad for k, v in leaves.items()}


@pytest.mark.parametrize("ts", [8, 16])
def test_blend_variants_agree(ts):
    p, cams = scene()
    w = torch.randn(640 * 480, 3, generator=torch.Generator().manual_seed(1)).to(DEV)
    try:
        set_blend_variant(0, 0)
        img0, g0 = render(p, cams, ts, w)
        assert float(img0.abs().sum()) > 0
        for f in (0, 1, 2):
            for b in (0, 1, 2):
                set_blend_variant(f, b)
                img, g = render(p, cams, ts, w)
                assert torch.equal(img, img0), (f, b)
                for k in g0:
                    rel = float((g[k] - g0[k]).norm() / g0[k].norm().clamp_min(1e-30))
                    assert rel < 1e-5, (f, b, k, rel)
    finally:
        set_blend_variant(0, 0)


def test_autotuner_on_the_gpu_leaves_its_choice_set():
    p, cams = scene()
    w = torch.ones(640 * 480, 3, device=DEV)
    try:
        tuner = TileAutotuner(warmup=1, reps=2)
        ts = tuner.pick("scene", lambda t: render(p, cams, t, w))
        cfg = tuner.choice("scene")
        assert cfg[0] == ts and get_blend_variant() == (cfg[1], cfg[2])
        assert len(tuner.timings("scene")) >= 3
    finally:
        set_blend_variant(0, 0)
