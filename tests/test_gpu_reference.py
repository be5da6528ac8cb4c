"""GPU parity against the reference itself: the reference's own CUDA kernels
(compiled from its sources into oracle/_ref by oracle/build_ref.py) and the
GB300 kernels run on identical inputs on the same GPU.

Bars: sorted intersection ids, flatten ids, tiles-per-primitive and offsets
bit-exact; images and alphas within 1e-5 max abs (FP32); gradients within 1e-4
relative (L2 per tensor) of the reference backward.
"""
import numpy as np
import pytest
import torch

import ref_gpu
from scenes import beta_params, intrinsics, look_at, orbit_camera, projected_scene, rest_indices

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_gpu.available(),
                                 reason="reference cubins not built (oracle/build_ref.py)")]
DEV = "cuda"


@pytest.fixture(scope="module")
def ref():
    return ref_gpu.RefKernels()


def rel_l2(a, b):
    a = a.detach().double()
    b = b.detach().double()
    return float((a - b).norm() / b.norm().clamp_min(1e-30))


def test_projection_matches_reference(ref):
    from gsplat.cuda._wrapper import fully_fused_projection
    g = torch.Generator().manual_seed(21)
    N, C, W, H = 20000, 2, 640, 480
    means = ((torch.rand(N, 3, generator=g) * 2 - 1) * 2).to(DEV)
    Lm = torch.randn(N, 3, 3, generator=g) * 0.03
    cov33 = (Lm @ Lm.transpose(1, 2) + 1e-4 * torch.eye(3)).to(DEV)
    c6 = cov33[:, [0, 0, 0, 1, 1, 2], [0, 1, 2, 1, 2, 2]].contiguous()
    vms = torch.stack([look_at((0.3, 0.2, -4.0)), orbit_camera(g, 4.0)]).to(DEV)
    Ks = torch.stack([intrinsics(500, 500, 320, 240)] * C).to(DEV)
    r_ref, m2_ref, d_ref, cn_ref, _ = ref.projection_fwd(means, c6, vms, Ks, W, H)
    radii, m2, d, cn, _ = fully_fused_projection(means, c6, None, None, vms, Ks, W, H)
    torch.cuda.synchronize()
    assert torch.equal(radii, r_ref), int((radii != r_ref).sum())
    v = r_ref > 0
    assert float((m2 - m2_ref)[v].abs().max()) <= 1e-4
    assert float((d - d_ref)[v].abs().max()) <= 1e-6
    assert rel_l2(cn[v], cn_ref[v]) < 1e-6
    gg = torch.Generator().manual_seed(22)
    vm2 = torch.randn(C, N, 2, generator=gg).to(DEV)
    vd = torch.randn(C, N, generator=gg).to(DEV)
    vcn = (torch.randn(C, N, 3, generator=gg) * 1e-2).to(DEV)
    vmeans_ref, vcov_ref, _ = ref.projection_bwd(means, c6, vms, Ks, W, H, 0.3, r_ref, cn_ref,
                                                 vm2, vd, vcn)
    mt = means.clone().requires_grad_(True)
    ct = c6.clone().requires_grad_(True)
    _, m2b, db, cnb, _ = fully_fused_projection(mt, ct, None, None, vms, Ks, W, H)
    ((m2b * vm2).sum() + (db * vd).sum() + (cnb * vcn).sum()).backward()
    assert rel_l2(mt.grad, vmeans_ref) < 1e-5
    assert rel_l2(ct.grad, vcov_ref) < 1e-5


@pytest.mark.parametrize("C,N,W,H", [(1, 30000, 1280, 720), (3, 8000, 640, 480)])
def test_isect_matches_reference_bit_exact(ref, C, N, W, H):
    from gsplat.cuda._wrapper import isect_offset_encode, isect_tiles
    s = projected_scene(N, W, H, C=C, seed=N, device=DEV)
    radii = s["radii"].clone()
    radii[:, ::13] = 0
    depths = s["depths"].clone()
    depths[:, ::7] = 2.5
    ts = 16
    tw, th = (W + ts - 1) // ts, (H + ts - 1) // ts
    tpg_r, ids_r, fl_r = ref.isect_tiles(s["means2d"], radii, depths, ts, tw, th)
    offs_r = ref.offset_encode(ids_r, C, tw, th)
    tpg, ids, fl = isect_tiles(s["means2d"], radii, depths, ts, tw, th)
    offs = isect_offset_encode(ids, C, tw, th)
    assert torch.equal(tpg, tpg_r)
    assert torch.equal(ids, ids_r)
    assert torch.equal(fl, fl_r)
    assert torch.equal(offs, offs_r)


@pytest.mark.parametrize("bg", [False, True])
def test_blend_matches_reference(ref, bg):
    from gsplat.cuda._wrapper import isect_offset_encode, isect_tiles, rasterize_to_pixels
    C, N, W, H, ts = 1, 20000, 800, 600, 16
    s = projected_scene(N, W, H, C=C, seed=77, device=DEV)
    tw, th = (W + ts - 1) // ts, (H + ts - 1) // ts
    _, ids, fl = isect_tiles(s["means2d"], s["radii"], s["depths"], ts, tw, th)
    offs = isect_offset_encode(ids, C, tw, th)
    bgs = torch.rand(C, 3, generator=torch.Generator().manual_seed(3)).to(DEV) if bg else None
    args = [s["means2d"], s["conics"], s["colors"], s["opacities"], s["betas"]]
    oc_r, oa_r, li_r = ref.raster_fwd(*args, bgs, W, H, ts, offs, fl)
    leaves = [a.clone().requires_grad_(True) for a in args]
    oc, oa = rasterize_to_pixels(*leaves, W, H, ts, offs, fl, backgrounds=bgs)
    torch.cuda.synchronize()
    assert float((oc - oc_r).abs().max()) < 1e-5
    assert float((oa - oa_r).abs().max()) < 1e-5
    gg = torch.Generator().manual_seed(5)
    wc = torch.randn(oc.shape, generator=gg).to(DEV)
    wa = torch.randn(oa.shape, generator=gg).to(DEV)
    ((oc * wc).sum() + (oa * wa).sum()).backward()
    refg = ref.raster_bwd(*args, bgs, W, H, ts, offs, fl, oa_r, li_r, wc, wa)
    for t, r, nm in zip(leaves, refg, ("means2d", "conics", "colors", "opacities", "betas")):
        assert rel_l2(t.grad, r) < 1e-4, (nm, rel_l2(t.grad, r))


@pytest.mark.parametrize("D", [6, 7])
def test_cond_and_covar_match_reference(ref, D):
    from gsplat.cuda import _wrapper as Wr
    N = 20000
    p = beta_params(N, D, seed=31, device=DEV)
    ri, rj = [t.to(DEV) for t in rest_indices(D)]
    scale = torch.nn.functional.softplus(p["scale"]).contiguous()
    l3 = p["l_triangle"][:, :3].contiguous()
    R_r = ref.rotmat_fwd(l3)
    cov_r = ref.covar_fwd(R_r, scale, p["l_triangle"], ri, rj)
    R = Wr.l_triangle_to_rotmat(l3)
    cov = Wr.rot_scale_l_triangle_to_covar(R, scale, p["l_triangle"], ri, rj)
    assert torch.equal(R, R_r)
    assert rel_l2(cov, cov_r) < 1e-6
    sp_r = ref.covar_fwd(R_r, scale, p["l_triangle"], ri, rj, spatial=True)
    sp = Wr.rot_scale_l_triangle_to_covar(R, scale, p["l_triangle"], ri, rj, spatial_block=True)
    assert rel_l2(sp, sp_r) < 1e-6
    vcov = torch.randn(cov.shape, generator=torch.Generator().manual_seed(1)).to(DEV)
    vr_r, vs_r, vl_r = ref.covar_bwd(R_r, scale, p["l_triangle"], ri, rj, vcov)
    Rl = R.detach().clone().requires_grad_(True)
    sl = scale.clone().requires_grad_(True)
    ll = p["l_triangle"].clone().requires_grad_(True)
    (Wr.rot_scale_l_triangle_to_covar(Rl, sl, ll, ri, rj) * vcov).sum().backward()
    assert rel_l2(Rl.grad, vr_r) < 1e-5 and rel_l2(sl.grad, vs_r) < 1e-5
    assert rel_l2(ll.grad, vl_r) < 1e-5
    assert torch.equal(ref.rotmat_bwd(vr_r.contiguous()),
                       torch.stack([vr_r[:, 0, 1] - vr_r[:, 1, 0], vr_r[:, 0, 2] - vr_r[:, 2, 0],
                                    vr_r[:, 1, 2] - vr_r[:, 2, 1]], -1))
    # conditioning
    means = torch.cat([p["xyz"], p["mean"]], 1).contiguous()
    opac = torch.sigmoid(p["opacity"]).contiguous()
    betas = (4 * torch.exp(p["beta"]))[:, 1:].contiguous()
    q = torch.nn.functional.normalize(p["xyz"] - torch.tensor([0.0, 0.0, -4.0], device=DEV), dim=-1)
    if D == 7:
        q = torch.cat([q, torch.full((N, 1), 0.3, device=DEV)], 1)
    q = q.contiguous()
    cov_c = cov_r.contiguous()
    om_r, oV_r, oo_r = ref.cond_fwd(means, cov_c, opac, betas, q)
    leaves = [t.clone().requires_grad_(True) for t in (means, cov_c, opac, betas)]
    prev = Wr.get_cond_grad_mode()
    Wr.set_cond_grad_mode("reference")
    try:
        om, oV, oo = Wr.cond_mean_convariance_opacity(*leaves, q)
        assert rel_l2(om, om_r) < 1e-6 and rel_l2(oV, oV_r) < 1e-6 and rel_l2(oo, oo_r) < 1e-5
        gg = torch.Generator().manual_seed(2)
        vm = torch.randn(N, 3, generator=gg).to(DEV)
        vV = torch.randn(N, 3, 3, generator=gg).to(DEV)
        vo = torch.randn(N, 1, generator=gg).to(DEV)
        ((om * vm).sum() + (oV * vV).sum() + (oo * vo).sum()).backward()
    finally:
        Wr.set_cond_grad_mode(prev)
    ref_g = ref.cond_bwd(means, cov_c, opac, betas, q, vm, vV, vo)
    for t, r, nm in zip(leaves, ref_g, ("means", "covars", "opacities", "betas")):
        assert rel_l2(t.grad, r) < 1e-4, (nm, rel_l2(t.grad, r))
