"""The viewer's per-frame render on the fused path.

BetaModel.view (scene/beta_model.py:725-831) renders one frame for the
interactive viewer: Beta quantile masks over the raw betas (torch.quantile,
i.e. a sort of each N-vector, every frame), conditioning of every primitive,
seven masked gathers, rasterization with the viewer's near / far / radius
clip, "Alpha" and "Depth" images through a depth colormap whose min / max
are read back to the host, then a copy of the frame to the host.

FrameRenderer.render does the same frame as: the quantile bounds by an exact
radix select on the device and one mask kernel (ubs_quantile_mask), the
fused render with that mask (masked primitives are skipped where they are
projected: no gathers, same image), the colormap on the device
(ubs_depth_colormap), and one copy into pinned memory -- the only wait of
the frame besides the render's intersection-count check.

`view(model, camera_state, render_tab_state)` is a drop-in for the method,
taking the same nerfview camera state (c2w, get_K) and BetaRenderTabState
fields (scene/beta_viewer.py:10-23).
"""
from dataclasses import dataclass
from typing import Optional, Tuple

import numpy as np
import torch

from . import _lib as L
from .render import Renderer, Views
from .scene import Camera

PARAM_NAMES = ("xyz", "mean", "scale", "l_triangle", "opacity", "beta", "rgb")


@dataclass
class ViewState:
    """The render controls of BetaRenderTabState (scene/beta_viewer.py:10-23)."""
    timestamp: float = 0.0
    near_plane: float = 1e-3
    far_plane: float = 1e3
    radius_clip: float = 0.0
    b_xyz: Tuple[float, float] = (0, 100)
    b_view: Tuple[float, float] = (0, 100)
    b_time: Tuple[float, float] = (0, 100)
    backgrounds: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    render_mode: str = "RGB"  # "RGB", "Alpha", "Depth", "Normal"


def colormap_table(name="turbo", device="cuda"):
    """The 256-entry colour table the reference indexes (matplotlib's
    colormaps[name].colors, utils/general_utils.py:191-194) when matplotlib is
    importable; otherwise a grey ramp, and callers wanting the reference's
    colours pass their own table to FrameRenderer."""
    try:
        from matplotlib import colormaps
        colors = colormaps[name].colors
        return torch.tensor(colors, dtype=torch.float32, device=device).reshape(256, 3)
    except Exception:  # noqa: BLE001 (matplotlib absent or without the map)
        ramp = torch.arange(256, dtype=torch.float32) / 255.0
        return ramp[:, None].expand(256, 3).contiguous().to(device)


class FrameRenderer:
    """Renders viewer frames of one scene.  Keep one per viewer (it holds the
    render workspace, the colour table and two pinned output buffers; the
    array a frame returns is overwritten two frames later unless copy=True)."""

    def __init__(self, dim: int = 6, tile_size: int = 16, table: Optional[torch.Tensor] = None,
                 device="cuda"):
        self.dim = dim
        self.device = torch.device(device)
        self.renderer = Renderer(dim=dim, tile_size=tile_size)
        self.table = (table if table is not None else colormap_table(device=self.device))
        self.table = self.table.to(self.device, torch.float32).contiguous()
        if self.table.shape != (256, 3):
            raise ValueError("the colour table must be [256, 3]")
        self._host = [None, None]
        self._ring = 0
        self._qws = None
        self._arrays = None
        self._mm = torch.empty(4, dtype=torch.int32, device=self.device)
        self.total_count = 0
        self.rendered_count = 0

    # ------------------------------------------------------------- pieces
    def quantile_mask(self, raw_beta: torch.Tensor, state: ViewState) -> torch.Tensor:
        """uint8 [N] mask of the primitives inside the state's Beta quantile
        ranges (quantile_mask, scene/beta_model.py:729-757): the tested
        arrays are formed as the reference forms them, the bounds and the
        mask by the library's radix select."""
        import ctypes
        N = raw_beta.shape[0]
        arrays = [raw_beta[:, 0], raw_beta[:, 1:4].mean(dim=-1)]
        q = [state.b_xyz[0] / 100, state.b_xyz[1] / 100, state.b_view[0] / 100,
             state.b_view[1] / 100]
        if self.dim == 7:
            arrays.append(raw_beta[:, 4])
            q += [state.b_time[0] / 100, state.b_time[1] / 100]
        ptrs = (ctypes.c_void_p * len(arrays))(*[a.data_ptr() for a in arrays])
        strides = (ctypes.c_int64 * len(arrays))(*[a.stride(0) for a in arrays])
        qa = (ctypes.c_double * len(q))(*q)
        mask = torch.empty(N, dtype=torch.uint8, device=raw_beta.device)
        if self._qws is None:
            self._qws = L.workspace(L.query("ubs_quantile_mask_workspace_bytes"),
                                    raw_beta.device)
        L.call("ubs_quantile_mask", N, len(arrays), ctypes.cast(ptrs, ctypes.c_void_p),
               ctypes.cast(strides, ctypes.c_void_p), ctypes.cast(qa, ctypes.c_void_p),
               L.ptr(mask), L.ptr(self._qws), self._qws.numel(), L.stream(raw_beta.device))
        self._arrays = arrays  # alive until the launches that read them are done
        return mask

    def colormap(self, image: torch.Tensor) -> torch.Tensor:
        """apply_depth_colormap (utils/general_utils.py:196-218) of a
        one-channel image [..., 1] -> [..., 3]."""
        img = image.contiguous()
        out = torch.empty(img.shape[:-1] + (3,), dtype=torch.float32, device=img.device)
        L.call("ubs_depth_colormap", L.ptr(img), img.numel(), L.ptr(self.table), L.ptr(out),
               L.ptr(self._mm), L.stream(img.device))
        return out

    # -------------------------------------------------------------- frame
    @torch.no_grad()
    def frame(self, params, c2w, K, width: int, height: int, state: ViewState):
        """One frame on the device: (image [H, W, 3], raw, visible) where raw
        is what the image was made from (RGB [H, W, 3], alpha or depth
        [H, W, 1]) and visible the count of rendered primitives (device)."""
        dev = self.device
        c2w = torch.as_tensor(np.asarray(c2w), dtype=torch.float32)
        K = torch.as_tensor(np.asarray(K), dtype=torch.float32)
        viewmat = torch.linalg.inv(c2w)
        cam = Camera(viewmat, K, int(width), int(height), timestamp=float(state.timestamp),
                     position=c2w[:3, 3])
        views = Views([cam], tile_size=self.renderer.tile_size, device=dev)
        mask = self.quantile_mask(params["beta"], state)
        mode = state.render_mode
        if mode not in ("RGB", "Alpha", "Depth", "Normal"):
            raise ValueError("render mode %r (RGB, Alpha, Depth, Normal)" % (mode,))
        r = self.renderer
        r.near, r.far, r.radius_clip = state.near_plane, state.far_plane, state.radius_clip
        if mode in ("Depth", "Normal"):
            bg = torch.zeros(1, 3, device=dev)
            color_mode = 1
        else:
            bg = (torch.tensor(state.backgrounds, dtype=torch.float32) / 255.0).to(dev)[None]
            color_mode = 0
        p = {k: params[k].detach() for k in PARAM_NAMES}
        colors, alphas, _, _, _ = r.forward_raw(p, views, bg, check=True, prim_mask=mask,
                                                color_mode=color_mode)
        H, W = int(height), int(width)
        if mode == "RGB":
            raw = colors.view(H, W, 3)
            img = raw
        elif mode == "Alpha":
            raw = alphas.view(H, W, 1)
            img = self.colormap(raw)
        elif mode == "Depth":
            raw = colors.view(H, W, 3)[..., :1]
            img = self.colormap(raw)
        else:
            from gsplat.utils import depth_to_normal
            raw = colors.view(H, W, 3)[..., :1]
            vm = viewmat.to(dev)[None]
            n = depth_to_normal(raw[None], torch.inverse(vm), K.to(dev)[None])
            img = ((n + 1) / 2)[0]
        N = p["xyz"].shape[0]
        self.total_count = N
        visible = (r.radii(views, N) > 0).sum()
        return img, raw, visible

    @torch.no_grad()
    def render(self, params, c2w, K, width: int, height: int, state: ViewState,
               copy: bool = False) -> np.ndarray:
        """One frame as a float32 [H, W, 3] host array: params are the raw
        scene tensors (xyz, mean, scale, l_triangle, opacity, beta, rgb), c2w
        the camera-to-world matrix and K the intrinsics of the viewer camera."""
        img, _, visible = self.frame(params, c2w, K, width, height, state)
        H, W = int(height), int(width)
        # the frame and the visible count to pinned host memory, one wait
        slot = self._ring
        self._ring ^= 1
        need = H * W * 3 + 1
        buf = self._host[slot]
        if buf is None or buf.numel() < need:
            buf = torch.empty(need, dtype=torch.float32, pin_memory=True)
            self._host[slot] = buf
        buf[:H * W * 3].view(H, W, 3).copy_(img, non_blocking=True)
        buf[H * W * 3:].copy_(visible.float().view(1), non_blocking=True)
        torch.cuda.current_stream(self.device).synchronize()
        self.rendered_count = int(buf[H * W * 3].item())
        out = buf[:H * W * 3].view(H, W, 3).numpy()
        return out.copy() if copy else out


def view(model, camera_state, render_tab_state, center=None):
    """Drop-in for BetaModel.view: renders the model's scene for a nerfview
    camera state and BetaRenderTabState, fills its count fields, returns the
    frame.  The FrameRenderer is kept on the model between frames."""
    tab = render_tab_state
    if getattr(tab, "preview_render", False):
        W, H = tab.render_width, tab.render_height
    else:
        W, H = tab.viewer_width, tab.viewer_height
    c2w = camera_state.c2w
    K = camera_state.get_K((W, H))
    fr = getattr(model, "_ubs_frames", None)
    if fr is None:
        fr = FrameRenderer(dim=model.input_dim)
        model._ubs_frames = fr
    if center:
        with torch.no_grad():
            model._xyz -= model._xyz.mean(dim=0, keepdim=True)
    state = ViewState(timestamp=getattr(tab, "timestamp", 0.0), near_plane=tab.near_plane,
                      far_plane=tab.far_plane, radius_clip=tab.radius_clip, b_xyz=tab.b_xyz,
                      b_view=tab.b_view, b_time=tab.b_time, backgrounds=tab.backgrounds,
                      render_mode=tab.render_mode)
    params = {"xyz": model._xyz, "mean": model._mean, "scale": model._scale,
              "l_triangle": model._l_triangle, "opacity": model._opacity, "beta": model._beta,
              "rgb": model._rgb}
    img = fr.render(params, c2w, K, W, H, state, copy=True)
    tab.total_count_number = fr.total_count
    tab.rendered_count_number = fr.rendered_count
    return img
