"""The blend's work counters (ubs_raster_pair_counts), which the benchmark's
roofline uses, against a plain per-pixel loop over the sorted records of a
small frame: contributing pairs, pairs a per-pixel loop evaluates up to
termination, and pairs up to each pixel's last contributor.  The loop runs
in float64, so a pixel whose termination decision sits within float32
rounding of the threshold may differ; the totals must agree to 1e-3."""
import ctypes

import numpy as np
import pytest
import torch

from ubs import _lib as L
from ubs import scene as S

pytestmark = pytest.mark.gpu
DEV = "cuda"
W, H, TS = 64, 48, 16


def test_pair_counts_match_a_per_pixel_loop():
    p = S.synthetic_params(3000, 6, seed=2, xyz_range=1.0, device=DEV)
    with torch.no_grad():
        p["scale"][:, :3] += 2.0
    cam = S.orbit_view(4, 3.0, W, H, 60.0, 60.0, device=DEV)
    ri, rj = S.rest_indices(6, DEV)
    bg = torch.zeros(3, device=DEV)
    with torch.no_grad():
        _, _, meta = S.render_view(p, cam, bg, ri, rj, tile_size=TS)
    m2, cn = meta["means2d"], meta["conics"]
    op, be = meta["opacities"].contiguous(), meta["betas"].contiguous()
    fl, offs = meta["flatten_ids"], meta["isect_offsets"]
    C, N = op.shape
    T = fl.numel()
    colors = p["rgb"].detach().expand(1, -1, -1).contiguous()
    ws = L.workspace(L.query("ubs_raster_workspace_bytes", T, 3), DEV)
    oc = torch.empty(1, H, W, 3, device=DEV)
    oa = torch.empty(1, H, W, 1, device=DEV)
    li = torch.empty(1, H, W, dtype=torch.int32, device=DEV)
    st = L.stream(DEV)
    L.call("ubs_raster_pack", C, N, 3, T, L.ptr(fl), L.ptr(m2), L.ptr(cn), L.ptr(op), L.ptr(be),
           L.ptr(colors), L.ptr(ws), ws.numel(), st)
    L.call("ubs_raster_fwd_packed", C, N, 3, T, L.ptr(colors), L.ptr(bg.view(1, 3)), None, W, H,
           TS, meta["tile_width"], meta["tile_height"], L.ptr(offs), L.ptr(oc), L.ptr(oa),
           L.ptr(li), 1, L.ptr(ws), ws.numel(), st)
    counts = (ctypes.c_uint64 * 3)()
    L.call("ubs_raster_pair_counts", L.ptr(ws), ctypes.cast(counts, ctypes.c_void_p), st)

    mx = m2[0].double().cpu().numpy()
    c3 = cn[0].double().cpu().numpy()
    o = op[0].double().cpu().numpy()
    b = be[0].double().cpu().numpy()
    ids = fl.cpu().numpy()
    off = offs[0].reshape(-1).cpu().numpy()
    tw = meta["tile_width"]
    contrib = evald = bwd = 0
    for py in range(H):
        for px in range(W):
            t = (py // TS) * tw + px // TS
            rs = off[t]
            re = off[t + 1] if t + 1 < off.size else T
            Tr, last, term = 1.0, -1, -1
            for k in range(rs, re):
                g = ids[k] % N
                dx, dy = mx[g, 0] - (px + 0.5), mx[g, 1] - (py + 0.5)
                sg = c3[g, 0] * dx * dx + c3[g, 2] * dy * dy + 2 * c3[g, 1] * dx * dy
                if sg < 0 or sg >= 1:
                    continue
                a = min(0.999, o[g] * (1 - sg) ** b[g])
                nt = Tr * (1 - a)
                if nt <= 1e-4:
                    term = k
                    break
                Tr, last = nt, k
                contrib += 1
            evald += (term - rs + 1) if term >= 0 else (re - rs)
            bwd += (last - rs + 1) if last >= 0 else 0
    got = [int(c) for c in counts]
    assert contrib > 10_000 and evald > contrib and bwd >= contrib
    for g_, w_ in zip(got, [contrib, evald, bwd]):
        assert abs(g_ - w_) <= 1e-3 * w_ + 2, (got, [contrib, evald, bwd])
