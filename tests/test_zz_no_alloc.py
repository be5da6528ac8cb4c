"""ubs_raster_fwd_noalloc (the forward blend on the library's fixed static
scratch) against ubs_raster_fwd (the same blend on a caller workspace), both
called through the C ABI on the same sorted intersections.

Two no-alloc calls run back to back, on different scenes, so the second reads
records the first one left in the shared scratch only if it failed to
overwrite them.  Tolerance as for the blend elsewhere: 1e-5 absolute on
colours and alphas, last_ids identical."""
import ctypes

import pytest
import torch

from scenes import projected_scene

pytestmark = pytest.mark.gpu
DEV = "cuda"
MAX_ISECTS = 524288  # UBS_RASTER_NOALLOC_MAX_ISECTS in include/ubs.h


def sorted_scene(N, W, H, seed, tile=16):
    from gsplat.cuda._wrapper import isect_offset_encode, isect_tiles
    s = projected_scene(N, W, H, seed=seed, device=DEV)
    tw, th = (W + tile - 1) // tile, (H + tile - 1) // tile
    _, isect_ids, flatten_ids = isect_tiles(s["means2d"], s["radii"], s["depths"], tile, tw, th)
    offsets = isect_offset_encode(isect_ids, 1, tw, th)
    bg = torch.tensor([[0.2, 0.1, 0.3]], device=DEV)
    return s, bg, offsets, flatten_ids.contiguous(), (W, H, tile, tw, th)


def outputs(W, H):
    return (torch.full((1, H, W, 3), float("nan"), device=DEV),
            torch.full((1, H, W), float("nan"), device=DEV),
            torch.full((1, H, W), -7, dtype=torch.int32, device=DEV))


def args(s, bg, offsets, fl, geom, outs):
    from ubs import _lib as L
    W, H, tile, tw, th = geom
    N = s["means2d"].shape[1]
    return [1, N, 3, fl.numel(), L.ptr(s["means2d"]), L.ptr(s["conics"]), L.ptr(s["colors"]),
            L.ptr(s["opacities"]), L.ptr(s["betas"]), L.ptr(bg), None, W, H, tile, tw, th,
            L.ptr(offsets), L.ptr(fl)] + [L.ptr(t) for t in outs]


def with_workspace(s, bg, offsets, fl, geom):
    from ubs import _lib as L
    W, H = geom[:2]
    outs = outputs(W, H)
    ws = L.workspace(L.query("ubs_raster_workspace_bytes", fl.numel(), 3), DEV)
    L.call("ubs_raster_fwd", *args(s, bg, offsets, fl, geom, outs), L.ptr(ws), ws.numel(),
           L.stream(DEV))
    return outs


def no_alloc(s, bg, offsets, fl, geom):
    from ubs import _lib as L
    W, H = geom[:2]
    outs = outputs(W, H)
    L.call("ubs_raster_fwd_noalloc", *args(s, bg, offsets, fl, geom, outs), L.stream(DEV))
    return outs


def test_no_alloc_matches_workspace_entry_point_twice():
    scenes = [sorted_scene(3000, 256, 192, seed=41), sorted_scene(2500, 200, 144, seed=42)]
    got = [no_alloc(*sc) for sc in scenes]  # two calls in a row on the shared scratch
    torch.cuda.synchronize()
    for sc, g in zip(scenes, got):
        assert 0 < sc[3].numel() <= MAX_ISECTS
        ref = with_workspace(*sc)
        torch.cuda.synchronize()
        assert float((g[0] - ref[0]).abs().max()) <= 1e-5
        assert float((g[1] - ref[1]).abs().max()) <= 1e-5
        assert torch.equal(g[2], ref[2])
        assert float(ref[1].mean()) > 0.1  # the scene covers the image


def test_no_alloc_rejects_more_than_its_scratch_holds():
    from ubs import _lib as L
    lib = L.lib()
    rc = lib.ubs_raster_fwd_noalloc(1, 10, 3, MAX_ISECTS + 1, *([None] * 7), 64, 64, 16, 4, 4,
                                    None, None, None, None, None, None)
    assert rc == -4  # UBS_ERR_OVERFLOW, before any device work
    assert "scratch limit" in L.last_error()
