"""ubs_raster_fwd_noalloc (the forward blend on the library's fixed static
scratch) against ubs_raster_fwd (the same blend on a caller workspace), both
called through the C ABI on the same sorted intersections.

Two no-alloc calls run back to back, on different scenes, so the second reads
records the first one left in the shared scratch only if it failed to
overwrite them.  Both record layouts are covered: packed colour records (3
channels, 48 bytes per intersection) and colours gathered in the kernel (8
channels, 32 bytes per intersection); so is a frame whose intersection count
is close to the scratch's limit.  Tolerance as for the blend elsewhere: 1e-5
absolute on colours and alphas, last_ids identical.  Device-side status (a
flatten index out of range) is read back through ubs_raster_noalloc_status."""
import ctypes

import pytest
import torch

from scenes import projected_scene

pytestmark = pytest.mark.gpu
DEV = "cuda"
MAX_ISECTS = 524288  # UBS_RASTER_NOALLOC_MAX_ISECTS in include/ubs.h
BAD_INDEX = 8        # device status bit: a flatten index outside [0, C*N)


def sorted_scene(N, W, H, seed, channels=3, tile=16):
    from gsplat.cuda._wrapper import isect_offset_encode, isect_tiles
    s = projected_scene(N, W, H, seed=seed, device=DEV)
    if channels != 3:
        g = torch.Generator().manual_seed(seed + 100)
        s["colors"] = torch.rand(1, N, channels, generator=g).to(DEV)
    tw, th = (W + tile - 1) // tile, (H + tile - 1) // tile
    _, isect_ids, flatten_ids = isect_tiles(s["means2d"], s["radii"], s["depths"], tile, tw, th)
    offsets = isect_offset_encode(isect_ids, 1, tw, th)
    bg = torch.linspace(0.1, 0.4, channels, device=DEV).view(1, channels)
    return s, bg, offsets, flatten_ids.contiguous(), (W, H, tile, tw, th)


def outputs(W, H, channels):
    return (torch.full((1, H, W, channels), float("nan"), device=DEV),
            torch.full((1, H, W), float("nan"), device=DEV),
            torch.full((1, H, W), -7, dtype=torch.int32, device=DEV))


def args(s, bg, offsets, fl, geom, outs):
    from ubs import _lib as L
    W, H, tile, tw, th = geom
    N, ch = s["colors"].shape[1], s["colors"].shape[2]
    return [1, N, ch, fl.numel(), L.ptr(s["means2d"]), L.ptr(s["conics"]), L.ptr(s["colors"]),
            L.ptr(s["opacities"]), L.ptr(s["betas"]), L.ptr(bg), None, W, H, tile, tw, th,
            L.ptr(offsets), L.ptr(fl)] + [L.ptr(t) for t in outs]


def with_workspace(s, bg, offsets, fl, geom):
    from ubs import _lib as L
    W, H = geom[:2]
    ch = s["colors"].shape[2]
    outs = outputs(W, H, ch)
    ws = L.workspace(L.query("ubs_raster_workspace_bytes", fl.numel(), ch), DEV)
    L.call("ubs_raster_fwd", *args(s, bg, offsets, fl, geom, outs), L.ptr(ws), ws.numel(),
           L.stream(DEV))
    return outs


def no_alloc(s, bg, offsets, fl, geom):
    from ubs import _lib as L
    W, H = geom[:2]
    outs = outputs(W, H, s["colors"].shape[2])
    L.call("ubs_raster_fwd_noalloc", *args(s, bg, offsets, fl, geom, outs), L.stream(DEV))
    return outs


def noalloc_status():
    from ubs import _lib as L
    st = ctypes.c_uint32(0)
    L.call("ubs_raster_noalloc_status", ctypes.byref(st), L.stream(DEV))
    return st.value


def check_same(sc, got):
    ref = with_workspace(*sc)
    torch.cuda.synchronize()
    assert float((got[0] - ref[0]).abs().max()) <= 1e-5
    assert float((got[1] - ref[1]).abs().max()) <= 1e-5
    assert torch.equal(got[2], ref[2])
    assert float(ref[1].mean()) > 0.1  # the scene covers the image


@pytest.mark.parametrize("channels", [3, 8])
def test_no_alloc_matches_workspace_entry_point_twice(channels):
    scenes = [sorted_scene(3000, 256, 192, seed=41, channels=channels),
              sorted_scene(2500, 200, 144, seed=42, channels=channels)]
    got = [no_alloc(*sc) for sc in scenes]  # two calls in a row on the shared scratch
    torch.cuda.synchronize()
    assert noalloc_status() == 0
    for sc, g in zip(scenes, got):
        assert 0 < sc[3].numel() <= MAX_ISECTS
        check_same(sc, g)


def test_no_alloc_near_its_limit():
    # a frame whose intersections fill most of the scratch (the primitive count
    # is reduced until the count fits)
    N = 120_000
    while True:
        sc = sorted_scene(N, 1024, 768, seed=43)
        if sc[3].numel() <= MAX_ISECTS:
            break
        N = int(N * 0.9 * MAX_ISECTS / sc[3].numel())
    assert sc[3].numel() > 0.75 * MAX_ISECTS
    got = no_alloc(*sc)
    torch.cuda.synchronize()
    check_same(sc, got)


def test_no_alloc_reports_a_bad_flatten_index():
    s, bg, offsets, fl, geom = sorted_scene(2000, 128, 96, seed=44)
    bad = fl.clone()
    bad[bad.numel() // 2] = s["colors"].shape[1] + 5  # outside [0, C*N): checked on the device
    no_alloc(s, bg, offsets, bad, geom)
    assert noalloc_status() & BAD_INDEX
    no_alloc(s, bg, offsets, fl, geom)  # the next call starts from a clear status
    assert noalloc_status() == 0


def test_no_alloc_rejects_more_than_its_scratch_holds():
    from ubs import _lib as L
    lib = L.lib()
    rc = lib.ubs_raster_fwd_noalloc(1, 10, 3, MAX_ISECTS + 1, *([None] * 7), 64, 64, 16, 4, 4,
                                    None, None, None, None, None, None)
    assert rc == -4  # UBS_ERR_OVERFLOW, before any device work
    assert "scratch limit" in L.last_error()
