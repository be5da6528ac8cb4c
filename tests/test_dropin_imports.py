"""The reference model's gsplat imports (scene/beta_model.py:12-22) resolve
against this package unchanged (import only: no device needed)."""


def test_beta_model_imports_resolve():
    from gsplat.rendering import rasterization
    from gsplat.cuda._torch_impl import (
        _l_triangle_to_rotmat,
        _rot_scale_l_triangle_to_covar,
        _cond_mean_convariance_opacity,
    )
    from gsplat.cuda._wrapper import (
        l_triangle_to_rotmat,
        rot_scale_l_triangle_to_covar,
        cond_mean_convariance_opacity,
    )
    import gsplat
    for name in gsplat.__all__:
        assert callable(getattr(gsplat, name)), name
    assert callable(rasterization) and callable(_l_triangle_to_rotmat)


def test_training_loss_imports_resolve():
    """train.py:17 and scene/__init__.py:26 import fused_ssim."""
    from fused_ssim import fused_ssim
    import inspect
    params = list(inspect.signature(fused_ssim).parameters)
    assert params == ["img1", "img2", "padding", "train"]
