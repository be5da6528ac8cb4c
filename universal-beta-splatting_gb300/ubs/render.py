"""Fused multi-view rendering of a Universal Beta Splatting scene (GB300 path).

One call renders a batch of views, of any mix of resolutions and timestamps,
with five stream-ordered launches (per-primitive forward, scan, emit, bucket
sort, blend) and one autograd node whose backward is two launches (blend
backward, per-primitive backward).  The mathematics is the reference model's
render (scene/beta_model.py:660-722 + rendering.py:17-232), evaluated per
(view, primitive): each primitive is conditioned on the ray to that view's
camera (and its timestamp), so views are consistent with rendering them one at
a time.

    from ubs.render import Renderer, Views
    r = Renderer(dim=6)
    views = Views([cam0, cam1], device="cuda")      # ubs.scene.Camera objects
    colors, alphas = r.render(params, views)       # flat [P, 3], [P]
    images = views.split(colors)                   # list of [H, W, 3]
"""
import ctypes
from typing import Dict, List, Optional, Sequence

import torch

from . import _lib as L

PARAM_ORDER = ("xyz", "mean", "scale", "l_triangle", "opacity", "beta", "rgb")
STATUS_OVERFLOW = 4
STATUS_NEG_DEPTH = 2


class Views:
    """Cameras of one render call, flattened into (view, tile) buckets and one
    pixel buffer.  `cameras` are ubs.scene.Camera objects (viewmat, K, width,
    height, timestamp).  The per-view tables go to the device in two copies
    from one pinned staging buffer, on `stream` (default: the current one)."""

    def __init__(self, cameras: Sequence, tile_size: int = 16, device=None, stream=None):
        if len(cameras) == 0:
            raise ValueError("need at least one view")
        device = torch.device(device or cameras[0].viewmat.device)
        C = len(cameras)
        fl = torch.empty(C * 24, dtype=torch.float32, pin_memory=torch.cuda.is_available())
        # int64 pix_base [C+1], then int32 dims [C,4] and tile_base [C+1]
        ints = torch.empty(2 * (C + 1) + 4 * C + C + 1, dtype=torch.int32,
                           pin_memory=torch.cuda.is_available())
        f = fl.view(C, 24)
        dims, tile_base, pix_base = [], [0], [0]
        for v, c in enumerate(cameras):
            vm = c.viewmat.detach().reshape(16).float().cpu()
            f[v, 0:16] = vm
            K = c.K.detach().float().cpu()
            f[v, 16:20] = torch.stack([K[0, 0], K[1, 1], K[0, 2], K[1, 2]])
            # the camera centre the reference model conditions on: the
            # camera's own value (computed where its matrices live), so the
            # view-direction queries round the same way
            center = getattr(c, "position", None)
            if center is None:
                center = getattr(c, "center", None)
            if center is not None:
                f[v, 20:23] = center.detach().reshape(3).float().cpu()
            else:
                R, t = vm.view(4, 4)[:3, :3], vm.view(4, 4)[:3, 3]
                f[v, 20:23] = -R.t() @ t
            f[v, 23] = float(c.timestamp)
            tw = (c.width + tile_size - 1) // tile_size
            th = (c.height + tile_size - 1) // tile_size
            dims.append([c.width, c.height, tw, th])
            tile_base.append(tile_base[-1] + tw * th)
            pix_base.append(pix_base[-1] + c.width * c.height)
        if tile_base[-1] >= 2 ** 31:
            raise ValueError("too many tiles in one render call")
        o = 2 * (C + 1)
        ints[:o].view(torch.int64)[:] = torch.tensor(pix_base, dtype=torch.int64)
        ints[o:o + 4 * C] = torch.tensor(dims, dtype=torch.int32).reshape(-1)
        ints[o + 4 * C:] = torch.tensor(tile_base, dtype=torch.int32)
        self.C = C
        self.tile_size = tile_size
        self.shapes = [(c.height, c.width) for c in cameras]
        self.n_buckets = tile_base[-1]
        self.n_pixels = pix_base[-1]
        self.pix_base_host = pix_base
        self.device = device
        if device.type == "cuda":
            st = stream if stream is not None else torch.cuda.current_stream(device)
            with torch.cuda.stream(st):
                fd = fl.to(device, non_blocking=True).view(C, 24)
                idev = ints.to(device, non_blocking=True)
                self.viewmats = fd[:, 0:16].contiguous()
                self.intr = fd[:, 16:20].contiguous()
                self.centers = fd[:, 20:23].contiguous()
                self.times = fd[:, 23].contiguous()
        else:  # host-side tables only (no compute runs on them)
            fd, idev = fl.clone().view(C, 24), ints.clone()
            self.viewmats, self.intr = fd[:, 0:16].contiguous(), fd[:, 16:20].contiguous()
            self.centers, self.times = fd[:, 20:23].contiguous(), fd[:, 23].contiguous()
        self._staging = (fl, ints)  # pinned buffers must outlive the copies
        self.pix_base = idev[:o].view(torch.int64)
        self.dims = idev[o:o + 4 * C].view(C, 4)
        self.tile_base = idev[o + 4 * C:]

    def split(self, flat: torch.Tensor) -> List[torch.Tensor]:
        """Per-view [H, W, ...] views of a flat per-pixel buffer."""
        out = []
        for v, (h, w) in enumerate(self.shapes):
            a, b = self.pix_base_host[v], self.pix_base_host[v + 1]
            out.append(flat[a:b].view(h, w, *flat.shape[1:]))
        return out

    def join(self, images: Sequence[torch.Tensor]) -> torch.Tensor:
        """Inverse of split: per-view [H, W, ...] tensors -> flat [P, ...]."""
        return torch.cat([im.reshape(-1, *im.shape[2:]) for im in images], 0)


class Renderer:
    """Renders scenes through the fused path and keeps the intersection
    capacity of its workspaces.  `exact_cond_grad` selects the exact
    conditioning gradient instead of the reference's backward formula."""

    def __init__(self, dim: int = 6, tile_size: int = 16, eps2d: float = 0.3,
                 near_plane: float = 0.01, far_plane: float = 1e10, radius_clip: float = 0.0,
                 capacity: Optional[int] = None, exact_cond_grad: bool = False):
        if dim not in (6, 7):
            raise ValueError("dim must be 6 or 7")
        self.dim = dim
        self.tile_size = tile_size
        self.eps2d, self.near, self.far, self.radius_clip = eps2d, near_plane, far_plane, radius_clip
        self.capacity = capacity
        self.exact_cond_grad = exact_cond_grad
        self.last_isects = None
        self._pending = None  # (pinned stats, event, capacity) of an unchecked frame
        self.last_ws, self.last_cap = None, None

    # ---------------------------------------------------------------- helpers
    def _check_pending(self):
        if self._pending is None:
            return
        stats, ev, cap = self._pending
        self._pending = None
        ev.synchronize()
        T, status = int(stats[0]), int(stats[1])
        self.last_isects = T
        if status & STATUS_NEG_DEPTH:
            raise RuntimeError("scene render: a visible primitive has a negative depth")
        if status & STATUS_OVERFLOW or T > cap:
            self.capacity = max(self.capacity or 0, int(T * 1.25) + 1024)
            raise RuntimeError("scene render: an earlier unchecked frame needed %d intersections "
                               "but had capacity %d; capacity is now %d" % (T, cap, self.capacity))

    def stats(self):
        """(intersections, status bits) of the last forward's workspace; raises
        if that frame overflowed its capacity.  Synchronises the stream."""
        import ctypes
        T, status = ctypes.c_int64(0), ctypes.c_uint32(0)
        L.call("ubs_scene_stats", L.ptr(self.last_ws), ctypes.byref(T), ctypes.byref(status),
               L.stream(self.last_ws.device))
        self.last_isects = int(T.value)
        if status.value & STATUS_NEG_DEPTH:
            raise RuntimeError("scene render: a visible primitive has a negative depth")
        if status.value & STATUS_OVERFLOW or T.value > self.last_cap:
            self.capacity = max(self.capacity or 0, int(T.value * 1.25) + 1024)
            raise RuntimeError("scene render: a frame needed %d intersections but had capacity "
                               "%d; capacity is now %d" % (T.value, self.last_cap, self.capacity))
        return int(T.value), int(status.value)

    def workspace_bytes(self, C, N, n_buckets, capacity):
        return L.query("ubs_scene_workspace_bytes", C, N, n_buckets, capacity)

    def radii(self, views: Views, N: int):
        """The last forward's per-(view, primitive) radii, int32 [C, N] (a view
        into its workspace; 0 where a primitive was not rendered)."""
        import ctypes
        r, d = ctypes.c_int64(), ctypes.c_int64()
        L.call("ubs_scene_workspace_offsets", views.C, N, views.n_buckets, self.last_cap,
               ctypes.byref(r), ctypes.byref(d))
        n = views.C * N
        return self.last_ws[r.value:r.value + 4 * n].view(torch.int32).view(views.C, N)

    def _sections(self, views: Views, N: int):
        """Byte offsets of the last forward's workspace sections
        (ubs_scene_workspace_layout: records, radii, depths, bucket starts,
        keys)."""
        secs = (ctypes.c_int64 * 5)()
        L.call("ubs_scene_workspace_layout", views.C, N, views.n_buckets, self.last_cap, secs, 5)
        return [int(x) for x in secs]

    def projected(self, views: Views, N: int):
        """The last forward's per-(view, primitive) projection, as the
        reference's meta entries: dict of means2d [C, N, 2], conics [C, N, 3],
        opacities [C, N] (conditioned), betas [C, N], radii int32 [C, N],
        depths [C, N] (views into the workspace; zeros where the radius is 0)."""
        rec, rad, dep, _, _ = self._sections(views, N)
        n = views.C * N
        r = self.last_ws[rec:rec + 32 * n].view(torch.float32).view(views.C, N, 8)
        return {"means2d": r[..., 0:2], "opacities": r[..., 2], "betas": r[..., 3],
                "conics": r[..., 4:7],
                "radii": self.last_ws[rad:rad + 4 * n].view(torch.int32).view(views.C, N),
                "depths": self.last_ws[dep:dep + 4 * n].view(torch.float32).view(views.C, N)}

    def intersections(self, views: Views, N: int):
        """The last forward's sorted intersections in the reference's layout,
        one entry per view: (isect_ids int64 [T_v] = tile << 32 | depth bits,
        flatten_ids int32 [T_v] = primitive index, isect_offsets int32
        [th, tw]) -- what isect_tiles + isect_offset_encode return for that
        view alone (isect_tiles.cu:82-96, 287-367).  Reads the intersection
        count (synchronises)."""
        T, _ = self.stats()
        _, _, _, o_off, o_key = self._sections(views, N)
        nb = views.n_buckets
        # bucket starts (exclusive scan of the counts); the end of the last
        # bucket is the intersection total
        starts = self.last_ws[o_off:o_off + 4 * nb].view(torch.int32).long()
        ends = torch.cat([starts[1:], starts.new_full((1,), T)])
        keys = self.last_ws[o_key:o_key + 8 * T].view(torch.int64)
        tb = views.tile_base.long().cpu()
        out = []
        for v in range(views.C):
            b0, b1 = int(tb[v]), int(tb[v + 1])
            a, b = int(starts[b0]), int(ends[b1 - 1])
            k = keys[a:b]
            counts = ends[b0:b1] - starts[b0:b1]
            tile = torch.repeat_interleave(torch.arange(b1 - b0, device=k.device), counts)
            ids = (tile << 32) | ((k >> 32) & 0xffffffff)
            fl = ((k & 0xffffffff) - v * N).to(torch.int32)
            h, w = views.shapes[v]
            ts = views.tile_size
            th, tw = (h + ts - 1) // ts, (w + ts - 1) // ts
            out.append((ids, fl, (starts[b0:b1] - a).to(torch.int32).view(th, tw)))
        return out

    def _args(self, p, views, bg):
        return [self.dim, p["xyz"].shape[0]] + [L.ptr(p[k]) for k in PARAM_ORDER] + [
            views.C, L.ptr(views.viewmats), L.ptr(views.intr), L.ptr(views.centers),
            L.ptr(views.times), L.ptr(views.dims), L.ptr(views.tile_base), L.ptr(views.pix_base),
            views.n_buckets, self.tile_size, float(self.eps2d), float(self.near), float(self.far),
            float(self.radius_clip), L.ptr(bg)]

    def forward_raw(self, p: Dict[str, torch.Tensor], views: Views, bg, check=True,
                    prim_mask=None, color_mode=0):
        """Run the forward kernels; returns (colors, alphas, last_ids, workspace, capacity).

        check=True reads the intersection count back (synchronising) and
        re-runs an overflowing frame; check=False reads it back
        asynchronously and reports an overflow at the next call; check="none"
        issues nothing but the kernels (safe inside CUDA graph capture) and
        leaves the verification to `stats()` after the frame(s).
        prim_mask (uint8 [N]) leaves out primitives whose entry is 0;
        color_mode=1 renders depth into channel 0 (one view, no backward)."""
        if check == "none":
            if self.capacity is None:
                raise RuntimeError("check='none' needs a capacity (render once with check=True)")
        else:
            self._check_pending()
        N = p["xyz"].shape[0]
        dev = p["xyz"].device
        # first frame: a guess from the pixel count (re-run below if too small)
        cap = self.capacity or max(1 << 16, min(16 * N * views.C, 8 * views.n_pixels))
        while True:
            ws = L.workspace(self.workspace_bytes(views.C, N, views.n_buckets, cap), dev)
            colors = torch.empty(views.n_pixels, 3, device=dev)
            alphas = torch.empty(views.n_pixels, device=dev)
            last = torch.empty(views.n_pixels, dtype=torch.int32, device=dev)
            st = L.stream(dev)
            if prim_mask is None and color_mode == 0:
                L.call("ubs_scene_forward", *self._args(p, views, bg), L.ptr(colors),
                       L.ptr(alphas), L.ptr(last), cap, L.ptr(ws), ws.numel(), st)
            else:
                L.call("ubs_scene_forward_masked", *self._args(p, views, bg), L.ptr(colors),
                       L.ptr(alphas), L.ptr(last), cap, L.ptr(ws), ws.numel(),
                       L.ptr(prim_mask, torch.uint8), int(color_mode), st)
            self.last_ws, self.last_cap = ws, cap
            if check == "none":
                return colors, alphas, last, ws, cap
            stats = torch.empty(2, dtype=torch.int64, pin_memory=True)
            hdr = ws[:16].view(torch.int64)
            if check:
                stats.copy_(hdr.cpu())
                T, status = int(stats[0]), int(stats[1]) & 0xffffffff
                self.last_isects = T
                if status & STATUS_NEG_DEPTH:
                    raise RuntimeError("scene render: a visible primitive has a negative depth")
                if T > cap:
                    cap = int(T * 1.25) + 1024
                    self.capacity = cap
                    continue
                if self.capacity is None:
                    self.capacity = max(int(T * 1.25) + 1024, 1 << 16)
            else:
                stats.copy_(hdr, non_blocking=True)
                ev = torch.cuda.Event()
                ev.record()
                self._pending = (stats, ev, cap)
            return colors, alphas, last, ws, cap

    def render(self, params: Dict[str, torch.Tensor], views: Views,
               backgrounds: Optional[torch.Tensor] = None, check=True):
        """Differentiable render of all views: colors [P, 3], alphas [P].
        `check`: True, False or "none", as for forward_raw."""
        dev = params["xyz"].device
        if backgrounds is None:
            bg = torch.zeros(views.C, 3, device=dev)
        else:
            bg = backgrounds.reshape(-1, 3).expand(views.C, 3).contiguous().float()
        tensors = [params[k] for k in PARAM_ORDER]
        return _SceneRender.apply(self, views, bg, check, *tensors)


def _prep(t, shape_tail=None):
    t = t.contiguous()
    if t.dtype != torch.float32:
        raise TypeError("scene parameters must be float32")
    return t


class _SceneRender(torch.autograd.Function):
    @staticmethod
    def forward(ctx, renderer, views, bg, check, xyz, mean, scale, l_triangle, opacity, beta, rgb):
        p = {"xyz": _prep(xyz), "mean": _prep(mean), "scale": _prep(scale),
             "l_triangle": _prep(l_triangle), "opacity": _prep(opacity.reshape(-1)),
             "beta": _prep(beta), "rgb": _prep(rgb)}
        colors, alphas, last, ws, cap = renderer.forward_raw(p, views, bg, check=check)
        ctx.renderer, ctx.views, ctx.ws, ctx.cap = renderer, views, ws, cap
        ctx.opacity_shape = opacity.shape
        ctx.save_for_backward(p["xyz"], p["mean"], p["scale"], p["l_triangle"], p["opacity"],
                              p["beta"], p["rgb"], bg, alphas, last)
        ctx.mark_non_differentiable(last)
        return colors, alphas

    @staticmethod
    def backward(ctx, v_colors, v_alphas):
        xyz, mean, scale, ltri, opac, beta, rgb, bg, alphas, last = ctx.saved_tensors
        r, views = ctx.renderer, ctx.views
        dev = xyz.device
        p = {"xyz": xyz, "mean": mean, "scale": scale, "l_triangle": ltri, "opacity": opac,
             "beta": beta, "rgb": rgb}
        v_colors = (torch.zeros(views.n_pixels, 3, device=dev) if v_colors is None
                    else v_colors.contiguous())
        v_alphas = (torch.zeros(views.n_pixels, device=dev) if v_alphas is None
                    else v_alphas.contiguous())
        g = {k: torch.empty_like(p[k]) for k in PARAM_ORDER}
        L.call("ubs_scene_backward", *r._args(p, views, bg), L.ptr(alphas), L.ptr(last),
               L.ptr(v_colors), L.ptr(v_alphas), *[L.ptr(g[k]) for k in PARAM_ORDER],
               int(bool(r.exact_cond_grad)), ctx.cap, L.ptr(ctx.ws), ctx.ws.numel(), L.stream(dev))
        ctx.ws = None
        return (None, None, None, None, g["xyz"], g["mean"], g["scale"], g["l_triangle"],
                g["opacity"].view(ctx.opacity_shape), g["beta"], g["rgb"])


class GraphedStep:
    """One training step -- fused render of `views`, `loss_fn(colors, alphas)`,
    backward to every parameter -- captured once into a CUDA graph and then
    replayed with a single launch.

    The parameters must keep their storage between replays (update them in
    place, e.g. with an optimizer or `copy_`); after each replay their `.grad`
    tensors (owned by the graph's memory pool) hold that step's gradients and
    `loss` holds its value.  The intersection capacity is fixed when the step
    is captured (the first frame's count times `headroom`); `check()` reads the
    last replay's count back and raises if the frame overflowed, in which case
    the step must be captured again.  Capture on parameter tensors that have
    not been through an eager backward on the default stream (or on fresh
    copies of them): PyTorch's gradient accumulation for such leaves would
    make the capture wait on that stream, which capture does not allow.

    With `optimizer` (ubs.optim.FusedAdam) the optimizer's update is captured
    too: the gradients then keep fixed storage (allocated while warming up,
    zeroed inside the graph) and `replay()` runs the optimizer's host part
    (`prepare()`) before launching the graph."""

    def __init__(self, renderer: Renderer, params: Dict[str, torch.Tensor], views: Views,
                 backgrounds: Optional[torch.Tensor], loss_fn, headroom: float = 1.5,
                 warmup: int = 3, before_capture=None, optimizer=None):
        self.r, self.p, self.views, self.loss_fn = renderer, params, views, loss_fn
        dev = params["xyz"].device
        self.bg = (torch.zeros(views.C, 3, device=dev) if backgrounds is None
                   else backgrounds.reshape(-1, 3).expand(views.C, 3).contiguous().float())
        with torch.no_grad():
            renderer.render(params, views, self.bg, check=True)
        renderer.capacity = int(renderer.last_isects * headroom) + 4096
        self.optimizer = optimizer
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            for _ in range(warmup):
                for v in params.values():
                    v.grad = None
                self._body()
                if optimizer is not None:
                    optimizer.step()
        torch.cuda.current_stream(dev).wait_stream(side)
        if optimizer is None:
            for v in params.values():
                v.grad = None
        if before_capture is not None:
            before_capture()
        self.graph = torch.cuda.CUDAGraph()
        n0 = L.query("ubs_launch_count")
        with torch.cuda.graph(self.graph):
            if optimizer is not None:
                for v in params.values():
                    v.grad.zero_()
            self.loss = self._body()
            if optimizer is not None:
                optimizer.launch()
        # library kernels in the graph (each replay launches them all)
        self.launches_per_replay = int(L.query("ubs_launch_count") - n0)

    def _body(self):
        colors, alphas = self.r.render(self.p, self.views, self.bg, check="none")
        loss = self.loss_fn(colors, alphas)
        loss.backward()
        return loss

    def replay(self):
        if self.optimizer is not None:
            self.optimizer.prepare()
        self.graph.replay()
        return self.loss

    def check(self):
        return self.r.stats()


class HostFedStep:
    """Steps whose inputs come from pinned host memory every step (a data
    loader, another process, a parameter store), with the copies of step k+1
    overlapping the compute of step k.

    `make_inputs()` returns (params, feeds, loss_fn): the parameter tensors
    of a GraphedStep, the device tensors that receive the host data each step
    (any of the parameters and, e.g., a target image the loss reads), and
    the loss over (colors, alphas).  It is called `depth` times (default 2):
    each buffer set gets its own tensors and its own captured step.
    `step(host)` copies host[i] (pinned, same shapes as feeds[i]) into the
    next set's feeds on a copy stream once that set's previous step is done,
    replays the set's graph on the current stream once the copies are done,
    and copies the loss into a pinned slot; `losses()` waits for the device
    and returns the values of the steps since the last call.  `start()` makes
    the copy stream wait for the current stream's work issued so far (call it
    where a timed region begins)."""

    def __init__(self, renderer: Renderer, views: Views, backgrounds, make_inputs,
                 depth: int = 2, headroom: float = 1.5, warmup: int = 3):
        if depth < 1:
            raise ValueError("depth must be >= 1")
        self.sets = []
        for _ in range(depth):
            params, feeds, loss_fn = make_inputs()
            gs = GraphedStep(renderer, params, views, backgrounds, loss_fn, headroom, warmup)
            self.sets.append((gs, list(feeds)))
        self.device = self.sets[0][1][0].device
        self.copy_stream = torch.cuda.Stream(self.device)
        self.copied = [torch.cuda.Event() for _ in range(depth)]
        self.done = [None] * depth
        self.ring = 256
        self.loss_host = torch.empty(self.ring, pin_memory=True)
        self.k = 0
        self.pending = []
        self.launches_per_step = self.sets[0][0].launches_per_replay

    def start(self):
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(self.device))
        self.copy_stream.wait_event(ev)

    def step(self, host: Sequence[torch.Tensor]):
        s = self.k % len(self.sets)
        gs, feeds = self.sets[s]
        if len(host) != len(feeds):
            raise ValueError("step() needs one host tensor per feed")
        cs = self.copy_stream
        cur = torch.cuda.current_stream(self.device)
        if self.done[s] is not None:
            cs.wait_event(self.done[s])  # the set's previous step has read its inputs
        with torch.cuda.stream(cs), torch.no_grad():
            for dst, src in zip(feeds, host):
                dst.copy_(src, non_blocking=True)
        self.copied[s].record(cs)
        cur.wait_event(self.copied[s])
        loss = gs.replay()
        slot = self.k % self.ring
        if len(self.pending) == self.ring:
            raise RuntimeError("call losses() at least every %d steps" % self.ring)
        self.loss_host[slot:slot + 1].copy_(loss.detach().view(1), non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(cur)
        self.done[s] = ev
        self.pending.append(slot)
        self.k += 1
        return slot

    def losses(self) -> List[float]:
        torch.cuda.current_stream(self.device).synchronize()
        out = [float(self.loss_host[i]) for i in self.pending]
        self.pending = []
        return out

    def check(self):
        return [gs.check() for gs, _ in self.sets]
