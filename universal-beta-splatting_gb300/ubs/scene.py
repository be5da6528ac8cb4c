"""A Universal Beta Splatting scene as plain tensors, and its render function.

`render_view` performs the same sequence of operator calls as the reference
model's render (scene/beta_model.py:660-722): activations, view-direction
query, rotation, D x D covariance, conditioning, then rasterization() — all
through the GB300 drop-in operators.  It exists so that benchmarks and tests
can drive the reference's call pattern without the reference's model class
(which needs plyfile / viser / sklearn).
"""
import math
from dataclasses import dataclass
from typing import Dict, Optional

import torch
import torch.nn.functional as F

from gsplat.cuda._wrapper import (cond_mean_convariance_opacity, l_triangle_to_rotmat,
                                  rot_scale_l_triangle_to_covar)
from gsplat.rendering import rasterization

PARAM_NAMES = ("xyz", "mean", "scale", "l_triangle", "opacity", "beta", "rgb")


def rest_indices(D: int, device=None):
    """Strictly-lower entries outside the 3x3 spatial block, row-major
    (scene/beta_model.py:69-73)."""
    ti, tj = torch.tril_indices(D, D, offset=-1)
    mask = (ti >= 3) | (tj >= 3)
    return (ti[mask].to(torch.int32).to(device), tj[mask].to(torch.int32).to(device))


@dataclass
class Camera:
    viewmat: torch.Tensor  # [4, 4] world-to-camera, row-major
    K: torch.Tensor  # [3, 3]
    width: int
    height: int
    timestamp: float = 0.0
    position: Optional[torch.Tensor] = None  # camera centre; default -R^T t of the viewmat

    @property
    def center(self) -> torch.Tensor:
        if self.position is not None:
            return self.position
        R = self.viewmat[:3, :3]
        t = self.viewmat[:3, 3]
        return -R.t() @ t


def synthetic_params(N: int, D: int = 6, seed: int = 0, xyz_range: float = 2.0,
                     device="cpu") -> Dict[str, torch.Tensor]:
    """Raw parameters with the benchmark's distributions: xyz uniform in
    [-r, r]^3, spatial scales exp(N(-4, 0.5)) (stored through the inverse
    softplus), angular scales ~1, rest lower-triangle N(0, 0.1), rotation skew
    N(0, 0.1), angular raw betas N(0, 0.5), spatial raw beta N(0, 0.3),
    opacity logits N(0, 1), RGB uniform [0, 1]; temporal mean uniform [0, 1]
    for D = 7."""
    g = torch.Generator().manual_seed(seed)
    K = D - 3
    xyz = (torch.rand(N, 3, generator=g) * 2 - 1) * xyz_range
    mean = torch.rand(N, K, generator=g) * 2 - 1
    if D == 7:
        mean[:, 3] = torch.rand(N, generator=g)
    s = torch.cat([torch.exp(torch.randn(N, 3, generator=g) * 0.5 - 4.0),
                   1.0 + 1e-5 * torch.randn(N, K, generator=g)], 1)
    scale = s + torch.log(-torch.expm1(-s))
    ltri = torch.randn(N, D * (D - 1) // 2, generator=g) * 0.1
    opacity = torch.randn(N, 1, generator=g)
    beta = torch.cat([torch.randn(N, 1, generator=g) * 0.3,
                      torch.randn(N, K, generator=g) * 0.5], 1)
    rgb = torch.rand(N, 3, generator=g)
    p = dict(xyz=xyz, mean=mean, scale=scale, l_triangle=ltri, opacity=opacity, beta=beta,
             rgb=rgb)
    return {k: v.to(device).contiguous() for k, v in p.items()}


def orbit_view(seed: int, radius: float, width: int, height: int, fx: float, fy: float,
               cx: Optional[float] = None, cy: Optional[float] = None, timestamp: float = 0.0,
               device="cpu") -> Camera:
    """Camera on a sphere of `radius` looking at the origin (up +y), OpenCV axes."""
    g = torch.Generator().manual_seed(seed)
    v = torch.randn(3, generator=g, dtype=torch.float64)
    eye = v / v.norm() * radius
    f = -eye / eye.norm()
    up = torch.tensor([0.0, 1.0, 0.0], dtype=torch.float64)
    r = torch.linalg.cross(f, up)
    if r.norm() < 1e-6:
        r = torch.linalg.cross(f, torch.tensor([1.0, 0.0, 0.0], dtype=torch.float64))
    r = r / r.norm()
    u = torch.linalg.cross(r, f)
    Rw = torch.stack([r, -u, f], 0)
    vm = torch.eye(4, dtype=torch.float64)
    vm[:3, :3] = Rw
    vm[:3, 3] = -Rw @ eye
    K = torch.tensor([[fx, 0.0, width / 2 if cx is None else cx],
                      [0.0, fy, height / 2 if cy is None else cy], [0.0, 0.0, 1.0]])
    return Camera(vm.float().to(device), K.to(device), width, height, timestamp)


def render_view(p: Dict[str, torch.Tensor], cam: Camera, background: torch.Tensor,
                rest_i: torch.Tensor, rest_j: torch.Tensor, render_mode: str = "RGB",
                tile_size: int = 16):
    """One view through the drop-in operators, in the order of the reference
    model's render.  Returns (image [3,H,W], meta)."""
    D = p["scale"].shape[1]
    scale = F.softplus(p["scale"])
    beta = 4.0 * torch.exp(p["beta"])
    view_dir = p["xyz"] - cam.center.unsqueeze(0)
    view_dir = view_dir / view_dir.norm(dim=-1, keepdim=True)
    if D == 6:
        query = view_dir
    elif D == 7:
        query = torch.cat([view_dir, torch.full((view_dir.shape[0], 1), cam.timestamp,
                                                device=view_dir.device)], -1)
    else:
        raise NotImplementedError("Only implemented for 6D or 7D query")
    R = l_triangle_to_rotmat(p["l_triangle"][:, :3])
    covar = rot_scale_l_triangle_to_covar(R, scale, p["l_triangle"], rest_i, rest_j)
    means_nd = torch.cat([p["xyz"], p["mean"]], dim=-1)
    opac = torch.sigmoid(p["opacity"])
    means, convs, opacities = cond_mean_convariance_opacity(means_nd, covar, opac, beta[:, 1:],
                                                            query)
    rgbs, alphas, meta = rasterization(
        means=means, l_triagnles=p["l_triangle"], scales=scale, opacities=opacities.squeeze(-1),
        betas=beta[:, 0], colors=p["rgb"], viewmats=cam.viewmat.unsqueeze(0),
        Ks=cam.K.unsqueeze(0), width=cam.width, height=cam.height,
        backgrounds=background.unsqueeze(0), render_mode=render_mode, covars=convs,
        tile_size=tile_size)
    return rgbs.permute(0, 3, 1, 2)[0], alphas, meta
