"""Host-side helpers of the reference's gsplat.utils used by the render modes
(submodules/gsplat/utils.py:44-132): back-projection of a depth map and
normals from its finite differences, in plain PyTorch."""
import torch
import torch.nn.functional as F
from torch import Tensor


def depth_to_points(depths: Tensor, camtoworlds: Tensor, Ks: Tensor,
                    z_depth: bool = True) -> Tensor:
    """World-space points [..., H, W, 3] of a depth map [..., H, W, 1]."""
    assert depths.shape[-1] == 1, depths.shape
    assert camtoworlds.shape[-2:] == (4, 4) and Ks.shape[-2:] == (3, 3)
    H, W = depths.shape[-3:-1]
    dev = depths.device
    x, y = torch.meshgrid(torch.arange(W, device=dev), torch.arange(H, device=dev),
                          indexing="xy")
    fx, fy = Ks[..., 0, 0], Ks[..., 1, 1]
    cx, cy = Ks[..., 0, 2], Ks[..., 1, 2]
    u = (x - cx[..., None, None] + 0.5) / fx[..., None, None]
    v = (y - cy[..., None, None] + 0.5) / fy[..., None, None]
    dirs_cam = torch.stack([u, v, torch.ones_like(u)], dim=-1)
    dirs = torch.einsum("...ij,...hwj->...hwi", camtoworlds[..., :3, :3], dirs_cam)
    origins = camtoworlds[..., :3, -1]
    if not z_depth:
        dirs = F.normalize(dirs, dim=-1)
    return origins[..., None, None, :] + depths * dirs


def depth_to_normal(depths: Tensor, camtoworlds: Tensor, Ks: Tensor,
                    z_depth: bool = True) -> Tensor:
    """Unit normals [..., H, W, 3] from central differences; 1-pixel border is 0."""
    p = depth_to_points(depths, camtoworlds, Ks, z_depth=z_depth)
    dx = p[..., 2:, 1:-1, :] - p[..., :-2, 1:-1, :]
    dy = p[..., 1:-1, 2:, :] - p[..., 1:-1, :-2, :]
    n = F.normalize(torch.cross(dx, dy, dim=-1), dim=-1)
    return F.pad(n, (0, 0, 1, 1, 1, 1), value=0.0)
