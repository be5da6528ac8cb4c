"""Generate golden vectors from the reference's own CPU-capable PyTorch code.

The reference ships no tests and no fixtures.  Its module
submodules/gsplat/cuda/_torch_impl.py runs on the CPU for every per-primitive
step of the rasteriser path (rotation, D x D covariance, conditioning,
projection) and for tile intersection / offset encoding.  This script imports
that module from a checkout of the reference, runs it on small seeded inputs and
stores inputs plus outputs (and autograd gradients) as .npz files next to this
script.  The blend has no CPU implementation in the reference (it needs the CUDA
extension and nerfacc), so blend parity is pinned on the GPU instead.

Usage:  python tests/golden/make_golden.py /path/to/reference
"""
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("UBS_REFERENCE_ROOT")
if not REF:
    sys.exit("usage: %s /path/to/reference (or set UBS_REFERENCE_ROOT)" % sys.argv[0])
sys.path.insert(0, os.path.join(REF, "submodules"))
from gsplat.cuda import _torch_impl as ti  # noqa: E402

torch.set_default_dtype(torch.float32)


def rest_indices(D):
    ti_, tj_ = torch.tril_indices(D, D, offset=-1)
    mask = (ti_ >= 3) | (tj_ >= 3)
    return ti_[mask].to(torch.int32), tj_[mask].to(torch.int32)


def save(name, **arrays):
    out = {k: (v.detach().cpu().numpy() if torch.is_tensor(v) else np.asarray(v))
           for k, v in arrays.items()}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name, {k: v.shape for k, v in out.items()})


def gen_prims(g, N, D):
    """Activated primitive parameters with the reference's distributions."""
    K = D - 3
    nl = D * (D - 1) // 2
    ltri = torch.randn(N, nl, generator=g) * 0.1
    s_sp = torch.exp(torch.randn(N, 3, generator=g) * 0.5 - 1.0)
    s_ang = 1.0 + 1e-5 * torch.randn(N, K, generator=g)
    scale = torch.cat([s_sp, s_ang], 1)
    xyz = torch.rand(N, 3, generator=g) * 2 - 1
    mean_ang = torch.rand(N, K, generator=g) * 2 - 1
    if D == 7:
        mean_ang[:, 3] = torch.rand(N, generator=g)
    opac = torch.sigmoid(torch.randn(N, 1, generator=g))
    beta = 4 * torch.exp(torch.randn(N, D - 2, generator=g) * 0.5)
    # keep the per-dimension damping away from its kink at beta == 4
    beta = torch.where((beta - 4).abs() < 1e-3, beta + 1e-2, beta)
    q = torch.nn.functional.normalize(torch.randn(N, 3, generator=g), dim=-1)
    if D == 7:
        q = torch.cat([q, torch.rand(N, 1, generator=g)], 1)
    return dict(ltri=ltri, scale=scale, xyz=xyz, mean_ang=mean_ang, opac=opac, beta=beta, query=q)


def golden_rotmat_covar(g):
    for D in (6, 7):
        N = 256
        p = gen_prims(g, N, D)
        ri, rj = rest_indices(D)
        ltri = p["ltri"].clone().requires_grad_(True)
        scale = p["scale"].clone().requires_grad_(True)
        R = ti._l_triangle_to_rotmat(ltri[:, :3])
        cov = ti._rot_scale_l_triangle_to_covar(R, scale, ltri, ri.long(), rj.long())
        v_cov = torch.randn(cov.shape, generator=g)
        # gradients of <v_cov, cov> with respect to rot, scale, l_triangle
        R_leaf = R.detach().clone().requires_grad_(True)
        cov2 = ti._rot_scale_l_triangle_to_covar(R_leaf, scale, ltri, ri.long(), rj.long())
        gR, gs, gl = torch.autograd.grad((cov2 * v_cov).sum(), [R_leaf, scale, ltri])
        cov_sp = ti._rot_scale_l_triangle_to_covar(R.detach(), scale.detach(), ltri.detach(),
                                                   ri.long(), rj.long(), spatial_block=True)
        v_R = torch.randn(N, 3, 3, generator=g)
        l3 = ltri.detach()[:, :3].clone().requires_grad_(True)
        (gl3,) = torch.autograd.grad((ti._l_triangle_to_rotmat(l3) * v_R).sum(), [l3])
        save("covar_d%d" % D, ltri=ltri, scale=scale, rest_i=ri, rest_j=rj, rot=R, covar=cov,
             covar_spatial=cov_sp, v_covar=v_cov, g_rot=gR, g_scale=gs, g_ltri=gl, v_rot=v_R,
             g_l3=gl3)


def golden_cond(g):
    for D in (6, 7):
        N = 256
        K = D - 3
        p = gen_prims(g, N, D)
        ri, rj = rest_indices(D)
        R = ti._l_triangle_to_rotmat(p["ltri"][:, :3])
        cov = ti._rot_scale_l_triangle_to_covar(R, p["scale"], p["ltri"], ri.long(), rj.long())
        means = torch.cat([p["xyz"], p["mean_ang"]], 1).requires_grad_(True)
        cov = cov.detach().requires_grad_(True)
        opac = p["opac"].clone().requires_grad_(True)
        betas = p["beta"][:, 1:].clone().requires_grad_(True)
        q = p["query"]
        m, V, o = ti._cond_mean_convariance_opacity(means, cov, opac, betas, q)
        vm = torch.randn(m.shape, generator=g)
        vV = torch.randn(V.shape, generator=g)
        vo = torch.randn(o.shape, generator=g)
        gm, gV, go, gb = torch.autograd.grad((m * vm).sum() + (V * vV).sum() + (o * vo).sum(),
                                             [means, cov, opac, betas])
        assert betas.shape[1] == K
        save("cond_d%d" % D, means=means, covars=cov, opac=opac, betas=betas, query=q,
             out_means=m, out_covars=V, out_opac=o, v_means=vm, v_covars=vV, v_opac=vo,
             g_means=gm, g_covars=gV, g_opac=go, g_betas=gb)


def look_at(eye, target, up=(0.0, 1.0, 0.0)):
    eye = torch.tensor(eye, dtype=torch.float32)
    f = torch.tensor(target, dtype=torch.float32) - eye
    f = f / f.norm()
    upv = torch.tensor(up, dtype=torch.float32)
    r = torch.linalg.cross(f, upv)
    r = r / r.norm()
    u = torch.linalg.cross(r, f)
    # OpenCV convention: x right, y down, z forward
    Rw2c = torch.stack([r, -u, f], 0)
    vm = torch.eye(4)
    vm[:3, :3] = Rw2c
    vm[:3, 3] = -Rw2c @ eye
    return vm


def golden_projection(g):
    N = 200
    W, H = 160, 120
    K = torch.tensor([[150.0, 0, 80.0], [0, 150.0, 60.0], [0, 0, 1]])
    vm = look_at((0.3, -0.2, -4.0), (0.0, 0.0, 0.0))
    # primitives in front of the camera, near the image centre, so that the
    # 1-sigma (CUDA) and 3-sigma (torch) validity tests agree on every one
    means = (torch.rand(N, 3, generator=g) * 2 - 1) * torch.tensor([0.6, 0.45, 0.8])
    L = torch.randn(N, 3, 3, generator=g) * 0.05
    cov33 = L @ L.transpose(1, 2) + 1e-3 * torch.eye(3)
    covars6 = cov33[:, [0, 0, 0, 1, 1, 2], [0, 1, 2, 1, 2, 2]]
    means = means.clone().requires_grad_(True)
    c6 = covars6.clone().requires_grad_(True)
    idx_r = [[0, 1, 2], [1, 3, 4], [2, 4, 5]]
    cov_full = c6[:, torch.tensor(idx_r)]
    radii, m2, d, cn, _ = ti._fully_fused_projection(means, cov_full, vm[None], K[None], W, H)
    assert bool((radii > 0).all()), "golden projection scene must keep every primitive"
    v_m2 = torch.randn(m2.shape, generator=g)
    v_d = torch.randn(d.shape, generator=g)
    v_cn = torch.randn(cn.shape, generator=g) * 1e-2
    gm, gc = torch.autograd.grad((m2 * v_m2).sum() + (d * v_d).sum() + (cn * v_cn).sum(),
                                 [means, c6])
    save("projection", means=means, covars6=c6, viewmats=vm[None], Ks=K[None], width=W,
         height=H, radii3=radii, means2d=m2, depths=d, conics=cn, v_means2d=v_m2, v_depths=v_d,
         v_conics=v_cn, g_means=gm, g_covars6=gc)


def golden_isect(g):
    C, N = 2, 150
    W, H, ts = 100, 72, 16
    tw, th = (W + ts - 1) // ts, (H + ts - 1) // ts
    means2d = torch.rand(C, N, 2, generator=g) * torch.tensor([W + 40.0, H + 40.0]) - 20.0
    radii = torch.randint(0, 30, (C, N), generator=g, dtype=torch.int32)
    radii[:, ::7] = 0
    depths = torch.rand(C, N, generator=g) * 5 + 0.1
    tpg, ids, fl = ti._isect_tiles(means2d, radii, depths, ts, tw, th)
    offs = ti._isect_offset_encode(ids, C, tw, th)
    save("isect", means2d=means2d, radii=radii, depths=depths, tile_size=ts, tile_width=tw,
         tile_height=th, tiles_per_gauss=tpg, isect_ids=ids, flatten_ids=fl, offsets=offs)


if __name__ == "__main__":
    g = torch.Generator().manual_seed(0)
    golden_rotmat_covar(g)
    golden_cond(g)
    golden_projection(g)
    golden_isect(g)
