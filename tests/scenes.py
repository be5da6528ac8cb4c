"""Seeded synthetic scenes shared by the tests (no dataset is available; these
stand in for the reference's scenes with its parameter distributions)."""
import math

import numpy as np
import torch


def rest_indices(D):
    """Row-major strictly-lower entries outside the 3x3 spatial block, as the
    reference model builds them (scene/beta_model.py:69-73)."""
    ti, tj = torch.tril_indices(D, D, offset=-1)
    mask = (ti >= 3) | (tj >= 3)
    return ti[mask].to(torch.int32), tj[mask].to(torch.int32)


def look_at(eye, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0)):
    """World-to-camera [4,4] (x right, y down, z forward)."""
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, np.float64))
    if np.linalg.norm(r) < 1e-8:
        r = np.cross(f, np.array([1.0, 0.0, 0.0]))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    R = np.stack([r, -u, f], 0)
    vm = np.eye(4)
    vm[:3, :3] = R
    vm[:3, 3] = -R @ eye
    return torch.tensor(vm, dtype=torch.float32)


def orbit_camera(gen, radius):
    v = torch.randn(3, generator=gen, dtype=torch.float64).numpy()
    v /= np.linalg.norm(v)
    return look_at(v * radius)


def intrinsics(fx, fy, cx, cy):
    return torch.tensor([[fx, 0, cx], [0, fy, cy], [0, 0, 1]], dtype=torch.float32)


def beta_params(N, D=6, seed=0, xyz_range=1.0, log_scale_mu=-4.0, log_scale_sigma=0.5,
                rest_sigma=0.1, device="cpu"):
    """Raw (pre-activation) parameters of a UBS model with N D-dimensional
    primitives, drawn like the benchmark configuration: xyz uniform, spatial
    scales exp(N(mu, sigma)) (through the inverse softplus), angular scales ~1,
    rest lower-triangle N(0, rest_sigma), angular raw betas N(0, 0.5), spatial
    raw beta N(0, 0.3), opacity logits N(0, 1), RGB uniform."""
    g = torch.Generator().manual_seed(seed)
    K = D - 3
    nl = D * (D - 1) // 2
    xyz = (torch.rand(N, 3, generator=g) * 2 - 1) * xyz_range
    mean = torch.rand(N, K, generator=g) * 2 - 1
    if D == 7:
        mean[:, 3] = torch.rand(N, generator=g)
    s_sp = torch.exp(torch.randn(N, 3, generator=g) * log_scale_sigma + log_scale_mu)
    s_ang = 1.0 + 1e-5 * torch.randn(N, K, generator=g)
    s = torch.cat([s_sp, s_ang], 1)
    scale = s + torch.log(-torch.expm1(-s))  # inverse softplus
    ltri = torch.randn(N, nl, generator=g) * rest_sigma
    ltri[:, :3] = torch.randn(N, 3, generator=g) * 0.1
    opacity = torch.randn(N, 1, generator=g)
    beta = torch.cat([torch.randn(N, 1, generator=g) * 0.3,
                      torch.randn(N, D - 3, generator=g) * 0.5], 1)
    rgb = torch.rand(N, 3, generator=g)
    out = dict(xyz=xyz, mean=mean, scale=scale, l_triangle=ltri, opacity=opacity, beta=beta,
               rgb=rgb)
    return {k: v.to(device) for k, v in out.items()}


def projected_scene(N, W, H, C=1, seed=0, device="cpu", big_frac=0.0):
    """Random already-projected primitives (means2d, conics, opacities, betas,
    colours, depths, radii) for blend tests."""
    g = torch.Generator().manual_seed(seed)
    m2 = torch.stack([torch.rand(C, N, generator=g) * (W + 20) - 10,
                      torch.rand(C, N, generator=g) * (H + 20) - 10], -1)
    a = torch.exp(torch.randn(C, N, generator=g) * 0.6 + math.log(6.0))
    b = torch.exp(torch.randn(C, N, generator=g) * 0.6 + math.log(6.0))
    if big_frac > 0:
        big = torch.rand(C, N, generator=g) < big_frac
        a = torch.where(big, a * 8, a)
        b = torch.where(big, b * 8, b)
    th = torch.rand(C, N, generator=g) * math.pi
    c, s = torch.cos(th), torch.sin(th)
    sxx = a * a * c * c + b * b * s * s
    sxy = (a * a - b * b) * c * s
    syy = a * a * s * s + b * b * c * c
    det = sxx * syy - sxy * sxy
    conics = torch.stack([syy / det, -sxy / det, sxx / det], -1)
    radii = torch.ceil(torch.sqrt(torch.maximum(sxx, syy)) * 1.0).to(torch.int32) + 1
    opac = torch.rand(C, N, generator=g) * 0.8 + 0.05
    betas = torch.exp(torch.randn(C, N, generator=g) * 0.5) * 1.5
    colors = torch.rand(C, N, 3, generator=g)
    depths = torch.rand(C, N, generator=g) * 8 + 0.5
    out = dict(means2d=m2, conics=conics, radii=radii, opacities=opac, betas=betas,
               colors=colors, depths=depths)
    return {k: v.to(device) for k, v in out.items()}
