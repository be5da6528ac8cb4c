"""Names of the reference's gsplat.cuda._torch_impl that its model imports.

scene/beta_model.py:13-17 imports _l_triangle_to_rotmat,
_rot_scale_l_triangle_to_covar and _cond_mean_convariance_opacity (the
PyTorch twins of the CUDA operators, submodules/gsplat/cuda/_torch_impl.py:
9-129) but never calls them.  So that the import succeeds unchanged, the same
names are provided here with the same arguments and results; they run the
GB300 CUDA operators of gsplat.cuda._wrapper (there is no CPU implementation
in this package).
"""
from torch import Tensor

from . import _wrapper as _W


def _cond_mean_convariance_opacity(means: Tensor, covars: Tensor, opacities: Tensor,
                                   betas: Tensor, query: Tensor):
    """Conditioned mean [N,3], covariance [N,3,3], opacity [N,1]."""
    return _W.cond_mean_convariance_opacity(means, covars, opacities, betas, query)


def _l_triangle_to_rotmat(l_triangle: Tensor) -> Tensor:
    """R = I + A from the first three entries of l_triangle [N, >=3]."""
    return _W.l_triangle_to_rotmat(l_triangle[:, :3])


def _rot_scale_l_triangle_to_covar(rot: Tensor, scale: Tensor, l_triangle: Tensor,
                                   rest_i: Tensor, rest_j: Tensor,
                                   spatial_block: bool = False) -> Tensor:
    """Sigma = L L^T, [N,D,D] (or its [N,3,3] spatial block)."""
    return _W.rot_scale_l_triangle_to_covar(rot, scale, l_triangle, rest_i, rest_j,
                                            spatial_block)
