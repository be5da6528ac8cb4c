#!/usr/bin/env python
"""Headline benchmark of the GB300 Universal Beta Splatting rasteriser.

Workload (the reference's plain GPU configuration): 1,000,000 6-D Beta
primitives (xyz uniform in [-2,2]^3, spatial scales exp(N(-4,0.5)), angular
scales ~1, rest lower-triangle N(0,0.1), angular raw betas N(0,0.5), spatial raw
beta N(0,0.3), opacity logits N(0,1), RGB uniform), one 1920x1080 pinhole camera
(fx=fy=1500) on a radius-4 orbit, 16x16 tiles.  One step = forward render of the
reference model's render (activations, rotation, covariance, conditioning,
projection, intersection + sort, blend), an L1 loss against a random target and
the backward pass to all raw parameters.  The headline runs the fused scene
render (ubs.render); the same step through the drop-in gsplat operators and
through the reference's own CUDA kernels (plain one-view-per-launch form) is
timed beside it.  Data are seeded synthetic tensors with the benchmark's
distributions (the reference's datasets are not available).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference path on the host CPU (the C++ oracle port
of every step; the reference itself has no CPU blend).  For N > 1 (torchrun)
each rank renders an independent replica (the path does not shard).
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "universal-beta-splatting_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402
import torch  # noqa: E402

METRIC = "render FPS and train it/s at 1M prims 1080p; serving p50/p99 ms vs plain form"
N_PRIMS, DIM, WIDTH, HEIGHT, FOCAL, TILE = 1_000_000, 6, 1920, 1080, 1500.0, 16
# Blend work for the roofline, counted from the reference's per-pair
# arithmetic (rasterize_to_pixels_fwd.cu:139-171, rasterize_to_pixels_bwd.cu:
# 158-247), 3 colour channels, no background.  FP32 FLOPs count a multiply or
# an add as 1 and an FMA as 2 (the FP32 probe's convention); comparisons,
# min/max and selects are not counted.  MUFU operations are counted apart and
# set against the XU pipe's own probe.
#   every pair a per-pixel loop evaluates: delta (2) + sigma (7 mul, 2 add) = 11
#   forward, per contributing pair: 1 - sigma, beta log2, opacity x, 1 - alpha,
#     T x, alpha T, 3 colour FMAs = 12 FLOPs; log2 + exp2 = 2 MUFU
#   backward, per contributing pair: alpha chain 4, T and fac 2, v_rgb 3,
#     v_alpha 15 + 3, v_sigma 5, v_conic 7, v_xy 10, v_opacity 1, v_beta 4,
#     colour buffer 6 = 60 FLOPs; log2, exp2 and two reciprocals (1 / (1 - alpha),
#     (1 - sigma)^(beta - 1) from the power) = 4 MUFU
# Units: the forward's evaluated pairs (up to the terminating record, else the
# tile's whole range) and the backward's pairs up to the last contributor --
# the hot-path scope table's units -- plus the contributing pairs of both.
PAIR_TEST_FLOP = 11
FWD_CONTRIB_FLOP, FWD_CONTRIB_MUFU = 12, 2
BWD_CONTRIB_FLOP, BWD_CONTRIB_MUFU = 60, 4
# FP32 operations per (pixel, channel) of the SSIM training loss and its
# gradient: two 11-tap passes (2 ops a tap) for the five windowed moments and
# for the three derivative maps, plus ~40 for the products, the map, its
# derivatives and the combine (utils/loss_utils.py:56-80, train.py:117-121)
LOSS_FLOP_PER_PX = 2 * 11 * (5 * 2 + 3 * 2) + 40
LOSS_BYTES_PER_PX = 12  # read the image and the target, write the gradient
LAMBDA_DSSIM = 0.2      # arguments/__init__.py
# learning rates of the reference's parameter groups (scene/beta_model.py:239-276)
TRAIN_LRS = {"xyz": 1.6e-4, "mean": 2e-3, "rgb": 2.5e-3, "opacity": 5e-2, "beta": 5e-3,
             "scale": 5e-3, "l_triangle": 1e-3}
WORKLOAD = ("1M 6-D Beta primitives, 1920x1080 (fx=fy=1500), radius-4 orbit camera, 16x16 tiles; "
            "forward + L1 loss + backward to all raw parameters, one view per step")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n-prims", type=int, default=N_PRIMS)
    ap.add_argument("--no-ref-gpu", action="store_true", help="skip timing the reference kernels")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the batched (C, D) and serving (E) configurations")
    ap.add_argument("--profile", action="store_true",
                    help="run only the fused step (capture, --warmup replays and one more) "
                         "for an ncu capture; prints no JSON line")
    ap.add_argument("--eager", action="store_true",
                    help="with --profile: launch the step kernel by kernel instead of a graph")
    ap.add_argument("--dropin", action="store_true",
                    help="with --profile: the step through the drop-in gsplat operators")
    ap.add_argument("--profile-config", choices=["C", "D"], default=None,
                    help="run only the batched step of config C or D (tile 16, default blend "
                         "variants: --warmup steps and one more) for an ncu capture; prints no "
                         "JSON line")
    ap.add_argument("--profile-neighbours", action="store_true",
                    help="run each training-step neighbour (Adam, the losses, MCMC, scene "
                         "file, viewer frame) once on the 1M scene for an ncu capture; prints "
                         "no JSON line")
    return ap.parse_args()


# --------------------------------------------------------------- utilities
class ClockSampler:
    """nvidia-smi clock / throttle samples every 200 ms while running."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.rows = []
        self.proc = None
        self.marks = {}

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append((time.time(), parts))

    def mark(self, name):
        self.marks[name] = time.time()

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self, t0, t1):
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        dev_index = None
        rows = [r for r in self.rows]
        if rows:
            dev_index = min(r[1][0] for r in rows)
            rows = [r for r in rows if r[1][0] == dev_index]
        inside = [r for r in rows if t0 <= r[0] <= t1]
        used = inside if len(inside) >= 3 else rows
        if not used:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm = [num(r[1][1]) for r in used if num(r[1][1]) is not None]
        mx = [num(r[1][2]) for r in used if num(r[1][2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in used for k in range(4)
                          if r[1][5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(used), "window": "timed region" if used is inside else "run"}


def replica_throughput(ms, world, device):
    """Whole-job step time and throughput of `world` independent replicas
    (the path does not shard: every rank runs the same per-rank workload):
    the job's step takes as long as its slowest rank."""
    ms_max = ms
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_max = float(t.item())
        dist.barrier()
    return ms_max, world * 1000.0 / ms_max


def l2_flush_buffer(dev):
    return torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)


# ------------------------------------------------------------- GPU (ours)
def make_problem(n_prims, seed, dev):
    from ubs import scene as S
    p = S.synthetic_params(n_prims, DIM, seed=seed, xyz_range=2.0, device=dev)
    for v in p.values():
        v.requires_grad_(True)
    cam = S.orbit_view(seed, 4.0, WIDTH, HEIGHT, FOCAL, FOCAL, device=dev)
    ri, rj = S.rest_indices(DIM, dev)
    bg = torch.zeros(3, device=dev)
    target = torch.rand(3, HEIGHT, WIDTH, generator=torch.Generator().manual_seed(seed + 7)).to(dev)
    return p, cam, ri, rj, bg, target


def gpu_step(p, cam, ri, rj, bg, target):
    from ubs import scene as S
    for v in p.values():
        v.grad = None
    img, _, meta = S.render_view(p, cam, bg, ri, rj, tile_size=TILE)
    loss = (img - target).abs().mean()
    loss.backward()
    return loss, meta


_SSIM_WIN = {}


def l1_loss(x, y):
    """The L1 term of the step through this library (one launch with its
    gradient, ubs.loss.l1_loss)."""
    from ubs.loss import l1_loss as _l1
    return _l1(x, y)


def torch_l1_ssim(img, gt, lam=LAMBDA_DSSIM):
    """train.py:117-121's loss on [N, 3, H, W] images with SSIM as
    utils/loss_utils.py:26-80 formulates it in PyTorch (F.conv2d, 11 x 11
    Gaussian window), the reference's own code for the SSIM term."""
    import torch.nn.functional as F
    c = img.shape[1]
    key = (c, img.device)
    if key not in _SSIM_WIN:
        d = torch.arange(11, dtype=torch.float64) - 5
        g = torch.exp(-d * d / (2 * 1.5 ** 2))
        g = (g / g.sum()).float()
        _SSIM_WIN[key] = (g[:, None] @ g[None, :]).expand(c, 1, 11, 11).contiguous().to(
            img.device)
    win = _SSIM_WIN[key]
    conv = lambda a: F.conv2d(a, win, padding=5, groups=c)  # noqa: E731
    mu1, mu2 = conv(img), conv(gt)
    s1, s2 = conv(img * img) - mu1 ** 2, conv(gt * gt) - mu2 ** 2
    s12 = conv(img * gt) - mu1 * mu2
    C1, C2 = 0.01 ** 2, 0.03 ** 2
    m = ((2 * mu1 * mu2 + C1) * (2 * s12 + C2)) / ((mu1 ** 2 + mu2 ** 2 + C1) * (s1 + s2 + C2))
    return (1.0 - lam) * (img - gt).abs().mean() + lam * (1.0 - m.mean())


class FusedStep:
    """One training step through the fused scene render: forward of the view,
    L1 loss against the target (or, with loss="l1_ssim_torch", the
    reference's full training loss in PyTorch), backward to all raw
    parameters."""

    def __init__(self, p, cam, bg, target, dev, loss="l1"):
        from ubs.render import Renderer, Views
        self.p = p
        self.renderer = Renderer(dim=DIM, tile_size=TILE)
        self.views = Views([cam], tile_size=TILE, device=dev)
        self.bg = bg.reshape(1, 3).contiguous()
        self.target = target.permute(1, 2, 0).reshape(-1, 3).contiguous()
        self.loss = loss
        self.hw = (cam.height, cam.width)
        self.target_nchw = target[None].contiguous()

    def prime(self):
        """First frame with a synchronous capacity check (sizes the buffers)."""
        with torch.no_grad():
            self.renderer.render(self.p, self.views, self.bg, check=True)

    def step(self):
        for v in self.p.values():
            v.grad = None
        colors, _ = self.renderer.render(self.p, self.views, self.bg, check=False)
        if self.loss == "l1":
            loss = l1_loss(colors, self.target)
        else:
            img = colors.view(1, self.hw[0], self.hw[1], 3).permute(0, 3, 1, 2)
            loss = torch_l1_ssim(img, self.target_nchw)
        loss.backward()
        return loss

    def forward(self):
        with torch.no_grad():
            self.renderer.render(self.p, self.views, self.bg, check=False)


def bench_loss(dev, flush, K):
    """The training loss and its gradient on one rendered 1920x1080 RGB image
    (the renderer's [1, H, W, 3] layout): the fused kernel against the
    PyTorch formulation of utils/loss_utils.py, and the kernel's roofline."""
    from ubs import _lib as L
    from ubs.loss import l1_ssim_loss
    g = torch.Generator().manual_seed(0)
    gt = torch.rand(1, HEIGHT, WIDTH, 3, generator=g)
    img = (gt + 0.05 * torch.randn(gt.shape, generator=g)).clamp(0, 1)
    gt, img = gt.to(dev), img.to(dev).requires_grad_(True)

    def ours():
        img.grad = None
        l1_ssim_loss(img, gt, LAMBDA_DSSIM, channels_last=True).backward()

    def plain():
        img.grad = None
        torch_l1_ssim(img.permute(0, 3, 1, 2), gt.permute(0, 3, 1, 2)).backward()

    for _ in range(3):
        ours()
        plain()
    t_ours = time_steps(ours, K, dev, flush)
    t_plain = time_steps(plain, K, dev, flush)
    L.profile_start(8 * (K + 1))
    for _ in range(K):
        flush.fill_(1.0)
        ours()
    torch.cuda.synchronize()
    prof = L.profile_stop()
    n_k, t_k = prof.get("ssim_map", (0, 0.0))
    n_g, t_g = prof.get("ssim_grad", (0, 0.0))
    k_ms = t_k / max(1, n_k) + t_g / max(1, n_g)  # the two launches of one loss
    px = HEIGHT * WIDTH * 3
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    fp32 = fp32_peak(dev)
    tflops = px * LOSS_FLOP_PER_PX / (k_ms * 1e-3) / 1e12 if k_ms else None
    gbs = px * LOSS_BYTES_PER_PX / (k_ms * 1e-3) / 1e9 if k_ms else None
    return {"ms": t_ours, "kernel_ms": k_ms,
            "map_kernel_ms": t_k / max(1, n_k), "grad_kernel_ms": t_g / max(1, n_g),
            "plain_pytorch_ms": t_plain,
            "speedup": t_plain / t_ours,
            "what": "0.8 L1 + 0.2 (1 - SSIM) and its backward on one 1920x1080x3 image: "
                    "one fused kernel (ubs.loss.l1_ssim_loss) vs the PyTorch formulation of "
                    "utils/loss_utils.py (F.conv2d, default cuDNN settings)",
            "roofline": {"bound": "fp32", "achieved": tflops, "peak": fp32, "unit": "TFLOP/s",
                         "frac": tflops / fp32 if (tflops and fp32) else None,
                         "algorithmic_work": "%d FP32 ops x %d pixel-channels" % (
                             LOSS_FLOP_PER_PX, px),
                         "hbm_gbs": gbs, "hbm_frac": gbs / peaks["hbm_gbs"]
                         if (gbs and peaks.get("hbm_gbs")) else None,
                         "hbm_bytes": px * LOSS_BYTES_PER_PX}}


def _torch_densify(m, cap_max, noise_factor):
    """The reference's densification step in PyTorch operations, for timing:
    relocation of dead primitives and addition of new ones
    (scene/beta_model.py:553-658) and the position noise (train.py:160-171),
    with the host synchronisations those operations imply (mask sum,
    nonzero, multinomial)."""
    names = ("xyz", "mean", "rgb", "opacity", "beta", "scale", "l_triangle")
    eps = torch.finfo(torch.float32).eps
    opt = m.optimizer

    def split(o_src, ratio):
        new = 1.0 - torch.pow(1.0 - o_src, 1.0 / (ratio + 1))
        new = torch.clamp(new, min=0.005, max=1.0 - eps)
        return torch.log(new / (1 - new))

    def draw(probs, num):
        pick = torch.multinomial(probs / (probs.sum() + eps), num, replacement=True)
        return pick

    with torch.no_grad():
        op = torch.sigmoid(m._opacity)
        dead = (op <= 0.005).squeeze(-1)
        if dead.sum() > 0:
            dead_idx = dead.nonzero(as_tuple=True)[0]
            alive_idx = (~dead).nonzero(as_tuple=True)[0]
            pick = alive_idx[draw(op[alive_idx, 0], dead_idx.shape[0])]
            ratio = torch.bincount(pick)[pick]
            new_op = split(op[pick, 0], ratio).unsqueeze(-1)
            for k in names:
                t = getattr(m, "_" + k)
                t.index_copy_(0, dead_idx, new_op if k == "opacity" else t[pick])
            m._opacity.index_copy_(0, pick, m._opacity.index_select(0, dead_idx))
            for k in names:
                st = opt.state[getattr(m, "_" + k)]
                st["exp_avg"][pick] = 0
                st["exp_avg_sq"][pick] = 0
        n = m._opacity.shape[0]
        n_add = max(0, min(cap_max, int(1.02 * n)) - n)
        if n_add > 0:
            op = torch.sigmoid(m._opacity)
            pick = draw(op[:, 0], n_add)
            ratio = torch.bincount(pick)[pick]
            new_op = split(op[pick, 0], ratio).unsqueeze(-1)
            new = {k: (new_op if k == "opacity" else getattr(m, "_" + k)[pick]) for k in names}
            m._opacity[pick] = new_op
            for group in opt.param_groups:
                k = group["name"]
                old = group["params"][0]
                st = opt.state.pop(old)
                st["exp_avg"] = torch.cat([st["exp_avg"], torch.zeros_like(new[k])])
                st["exp_avg_sq"] = torch.cat([st["exp_avg_sq"], torch.zeros_like(new[k])])
                st["exp_avg"][pick] = 0
                st["exp_avg_sq"][pick] = 0
                p = torch.nn.Parameter(torch.cat([old, new[k]]).requires_grad_(True))
                group["params"][0] = p
                opt.state[p] = st
                setattr(m, "_" + k, p)
        # position noise with the spatial covariance R diag(s^2) R^T
        s3 = torch.nn.functional.softplus(m._scale[:, :3])
        l = m._l_triangle[:, :3]
        one = torch.ones_like(l[:, 0])
        R = torch.stack([one, l[:, 0], l[:, 1], -l[:, 0], one, l[:, 2], -l[:, 1], -l[:, 2],
                         one], -1).view(-1, 3, 3)
        M = R * s3[:, None, :]
        cov = M @ M.transpose(1, 2)
        noise = torch.randn_like(m._xyz) * torch.pow(1 - torch.sigmoid(m._opacity), 100) \
            * noise_factor
        m._xyz.add_(torch.bmm(cov, noise.unsqueeze(-1)).squeeze(-1))


def bench_densify(p, dev, reps=5):
    """One MCMC densification step (relocate + add + position noise) on the
    1M-primitive scene with 10% dead primitives and Adam state: the device
    sequence (ubs.mcmc) against the PyTorch operations of the reference, wall
    clock per call with the device drained on both sides (the reference's
    operations synchronise in the middle)."""
    import time
    import types
    from ubs import mcmc
    names = ("xyz", "mean", "rgb", "opacity", "beta", "scale", "l_triangle")
    src = {"xyz": p["xyz"], "mean": p["mean"], "rgb": p["rgb"], "opacity": p["opacity"],
           "beta": p["beta"], "scale": p["scale"], "l_triangle": p["l_triangle"]}
    g = torch.Generator(device="cpu").manual_seed(0)
    dead_rows = torch.rand(src["opacity"].shape[0], generator=g) < 0.1

    def fresh():
        m = types.SimpleNamespace()
        groups = []
        for k in names:
            t = src[k].detach().clone().reshape(src[k].shape[0], -1)
            if k == "opacity":
                t[dead_rows.to(t.device)] = -8.0
            prm = torch.nn.Parameter(t)
            setattr(m, "_" + k, prm)
            groups.append({"params": [prm], "lr": 1e-3, "name": k})
        m.optimizer = torch.optim.Adam(groups, lr=0.0, eps=1e-15)
        for k in names:
            prm = getattr(m, "_" + k)
            st = m.optimizer.state[prm]
            st["step"] = torch.tensor(1.0)
            st["exp_avg"] = torch.zeros_like(prm)
            st["exp_avg_sq"] = torch.zeros_like(prm)
        torch.cuda.synchronize()
        return m

    cap = 10 ** 9
    factor = 1.0 * 1.6e-4

    def ours(m):
        mcmc.relocate_gs(m)
        mcmc.add_new_gs(m, cap)
        mcmc.perturb_xyz(m, factor)

    res = {}
    for name, fn in (("ours", ours), ("pytorch", lambda m: _torch_densify(m, cap, factor))):
        fn(fresh())  # warm-up
        ts = []
        for _ in range(reps):
            m = fresh()
            t0 = time.perf_counter()
            fn(m)
            torch.cuda.synchronize()
            ts.append((time.perf_counter() - t0) * 1e3)
            del m
        res[name] = sorted(ts)[len(ts) // 2]
    return {"ms": res["ours"], "plain_pytorch_ms": res["pytorch"],
            "speedup": res["pytorch"] / res["ours"],
            "what": "one MCMC densification step on 1M primitives with 10%% dead and Adam "
                    "state: relocation, +2%% addition, position noise; device kernels "
                    "(ubs.mcmc, no host synchronisation) vs the reference's PyTorch "
                    "operations (scene/beta_model.py:553-658, train.py:160-171); median "
                    "wall clock of %d calls" % reps}


def bench_scene_file(p, dev, reps=3):
    """Save and load of the 1M-primitive scene in the reference's PLY format:
    this library (native header/body I/O, chunked pinned copies, one
    pack/unpack kernel) against the reference's load_ply steps
    (scene/beta_model.py:322-404: per-property gathers into float64 arrays,
    then one torch.tensor(..., device="cuda") per parameter) with plyfile's
    binary read replaced by numpy's structured read (plyfile is not installed
    here).  The file sits in /tmp (page cache); median wall clock."""
    import tempfile
    import time
    from ubs import ply
    path = os.path.join(tempfile.gettempdir(), "ubs_bench_scene_%d_%d.ply" % (
        os.getpid(), int(os.environ.get("RANK", "0"))))
    names = ("xyz", "mean", "rgb", "opacity", "beta", "scale", "l_triangle")

    def ref_load():
        n, props, off = ply.read_header(path)
        rec = np.fromfile(path, dtype=[(nm, "<f4") for nm in props], offset=off, count=n)

        def fam(prefix):
            sel = sorted([nm for nm in props if nm.startswith(prefix)],
                         key=lambda s: int(s.split("_")[-1]))
            out = np.zeros((n, len(sel)))
            for i, nm in enumerate(sel):
                out[:, i] = np.asarray(rec[nm])
            return out

        xyz = np.stack((np.asarray(rec["x"]), np.asarray(rec["y"]), np.asarray(rec["z"])), 1)
        rgb = np.zeros((n, 3))
        for i, nm in enumerate(("red", "green", "blue")):
            rgb[:, i] = np.asarray(rec[nm])
        arrays = {"xyz": xyz, "mean": fam("mean_"), "rgb": rgb,
                  "opacity": np.asarray(rec["opacity"])[..., None], "beta": fam("beta_"),
                  "scale": fam("scale_"), "l_triangle": fam("l_triangle")}
        return {k: torch.tensor(arrays[k], dtype=torch.float, device=dev) for k in names}

    def med(fn):
        ts = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append((time.perf_counter() - t0) * 1e3)
        return sorted(ts)[len(ts) // 2]

    try:
        save_ms = med(lambda: ply.save_ply(path, p))
        load_ms = med(lambda: ply.load_ply(path, dev))
        ref_ms = med(ref_load)
        q = ply.load_ply(path, dev)
        r = ref_load()
        same = all(torch.equal(q[k], r[k]) for k in names)
        size = os.path.getsize(path)
    finally:
        if os.path.exists(path):
            os.remove(path)
    return {"save_ms": save_ms, "load_ms": load_ms, "reference_steps_load_ms": ref_ms,
            "load_speedup": ref_ms / load_ms, "file_bytes": size, "identical": same,
            "load_gbs": size / (load_ms * 1e-3) / 1e9,
            "what": "1M-primitive 6-D scene file (reference PLY layout): save and load "
                    "through ubs.ply vs the reference's load_ply steps with numpy's "
                    "structured read standing in for plyfile; median of %d" % reps}


def bench_viewer(p, cam, dev, reps=10):
    """Viewer frames of the 1M-primitive scene at 1920x1080 with Beta
    quantile ranges (5-95 % spatial, 5-95 % view): ubs.viewer.FrameRenderer
    against the steps of the reference's BetaModel.view
    (scene/beta_model.py:725-831: torch.quantile masks, conditioning, masked
    gathers, rasterization(), torch depth colormap, .cpu()) run on this
    library's drop-in operators; wall clock per frame to a host array."""
    import time
    import torch.nn.functional as F
    from gsplat.cuda._wrapper import (cond_mean_convariance_opacity, l_triangle_to_rotmat,
                                      rot_scale_l_triangle_to_covar)
    from gsplat.rendering import rasterization
    from ubs import scene as S
    from ubs.viewer import FrameRenderer, ViewState
    c2w = torch.inverse(cam.viewmat.cpu()).numpy()
    K = cam.K.cpu().numpy()
    table = torch.rand(256, 3, generator=torch.Generator().manual_seed(0)).to(dev)
    ri, rj = S.rest_indices(DIM, dev)

    def steps(mode):
        st = ViewState(b_xyz=(5, 95), b_view=(5, 95), render_mode=mode)
        c2w_t = torch.from_numpy(c2w).float().to(dev)
        K_t = torch.from_numpy(K).float().to(dev)
        beta_raw = p["beta"]
        x, v = beta_raw[:, 0], beta_raw[:, 1:4].mean(dim=-1)
        mask = ((x >= x.quantile(0.05)) & (x <= x.quantile(0.95)) & (v >= v.quantile(0.05))
                & (v <= v.quantile(0.95)))
        vd = p["xyz"] - c2w_t[:3, 3][None]
        q = vd / vd.norm(dim=-1, keepdim=True)
        scale = F.softplus(p["scale"])
        beta = 4.0 * torch.exp(p["beta"])
        R = l_triangle_to_rotmat(p["l_triangle"][:, :3])
        cov = rot_scale_l_triangle_to_covar(R, scale, p["l_triangle"], ri, rj)
        means, convs, opac = cond_mean_convariance_opacity(
            torch.cat([p["xyz"], p["mean"]], -1), cov, torch.sigmoid(p["opacity"]), beta[:, 1:],
            q)
        bg = torch.tensor(st.backgrounds, device=dev) / 255.0
        rc, ra, meta = rasterization(
            means=means[mask], l_triagnles=p["l_triangle"][mask], scales=scale[mask],
            opacities=opac.squeeze()[mask], betas=beta[:, :1].squeeze()[mask],
            colors=p["rgb"][mask], viewmats=torch.linalg.inv(c2w_t)[None], Ks=K_t[None],
            width=WIDTH, height=HEIGHT, backgrounds=bg[None], render_mode=mode,
            covars=convs[mask], near_plane=st.near_plane, far_plane=st.far_plane)
        int((meta["radii"] > 0).sum().item())
        if rc.shape[-1] == 1:
            near, far = float(torch.min(rc)), float(torch.max(rc))
            d = torch.nan_to_num(torch.clip((rc - near) / (far - near + 1e-10), 0.0, 1.0), 0)
            rc = table[(d * 255).long()[..., 0]]
        return rc[0].cpu().numpy()

    fr = FrameRenderer(dim=DIM, table=table)

    def ours(mode):
        st = ViewState(b_xyz=(5, 95), b_view=(5, 95), render_mode=mode)
        return fr.render(p, c2w, K, WIDTH, HEIGHT, st)

    def med(fn):
        fn()
        fn()
        ts = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            ts.append((time.perf_counter() - t0) * 1e3)
        return sorted(ts)[len(ts) // 2]

    with torch.no_grad():
        res = {"rgb_ms": med(lambda: ours("RGB")), "depth_ms": med(lambda: ours("Depth")),
               "steps_rgb_ms": med(lambda: steps("RGB")),
               "steps_depth_ms": med(lambda: steps("Depth"))}
    res["rgb_speedup"] = res["steps_rgb_ms"] / res["rgb_ms"]
    res["depth_speedup"] = res["steps_depth_ms"] / res["depth_ms"]
    res["what"] = ("viewer frame, 1M primitives, 1920x1080, Beta quantile ranges 5-95 %%, to a "
                   "host float32 array: ubs.viewer vs the reference's view() steps on the "
                   "drop-in operators; median wall clock of %d frames" % reps)
    return res


def profile_neighbours(p, cam, dev):
    """One run of each training-step neighbour on the headline scene, for
    ncu: Adam over the seven groups, the L1 + SSIM loss and the L1 loss on a
    1920x1080 image, MCMC relocation / addition / noise, a scene-file save
    and load, and viewer frames (RGB and Depth with quantile masks)."""
    import tempfile
    import types
    from ubs import mcmc, ply
    from ubs.loss import l1_loss as _l1, l1_ssim_loss
    from ubs.optim import FusedAdam
    from ubs.viewer import FrameRenderer, ViewState
    names = ("xyz", "mean", "rgb", "opacity", "beta", "scale", "l_triangle")
    g = torch.Generator(device="cpu").manual_seed(0)
    m = types.SimpleNamespace()
    for k in names:
        t = p[k].detach().clone().reshape(p[k].shape[0], -1)
        if k == "opacity":
            t[torch.rand(t.shape[0], generator=g).to(dev) < 0.1] = -8.0
        setattr(m, "_" + k, torch.nn.Parameter(t))
    m.optimizer = FusedAdam([{"params": [getattr(m, "_" + k)], "lr": TRAIN_LRS[k], "name": k}
                             for k in names], lr=0.0, eps=1e-15)
    for _ in range(2):
        for k in names:
            prm = getattr(m, "_" + k)
            prm.grad = torch.randn(prm.shape, device=dev) * 1e-3
        m.optimizer.step()
    gt = torch.rand(1, HEIGHT, WIDTH, 3, generator=g).to(dev)
    img = (gt + 0.05 * torch.randn(gt.shape, generator=g).to(dev)).clamp(0, 1).requires_grad_(True)
    l1_ssim_loss(img, gt, LAMBDA_DSSIM, channels_last=True).backward()
    img.grad = None
    _l1(img, gt).backward()
    mcmc.relocate_gs(m)
    mcmc.add_new_gs(m, 10 ** 9)
    mcmc.perturb_xyz(m, 1.6e-4)
    path = os.path.join(tempfile.gettempdir(), "ubs_profile_scene_%d.ply" % os.getpid())
    try:
        ply.save_ply(path, p)
        ply.load_ply(path, dev)
    finally:
        if os.path.exists(path):
            os.remove(path)
    fr = FrameRenderer(dim=DIM, table=torch.rand(256, 3, generator=g).to(dev))
    c2w = torch.inverse(cam.viewmat.cpu()).numpy()
    for mode in ("RGB", "Depth"):
        fr.render(p, c2w, cam.K.cpu().numpy(), WIDTH, HEIGHT,
                  ViewState(b_xyz=(5, 95), b_view=(5, 95), render_mode=mode))
    torch.cuda.synchronize()
    print("profile run (training-step neighbours)", flush=True)


def time_steps(fn, K, dev, flush, after=None):
    """Per-step CUDA-event time (ms), L2 flushed before every step (untimed);
    `after` runs after each step, outside the timed events."""
    total = 0.0
    for k in range(K):
        flush.fill_(float(k))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        total += e0.elapsed_time(e1)
        if after is not None:
            after()
    return total / K


def fp32_peak(dev):
    from ubs import _lib as L
    import ctypes
    ws = L.workspace(L.query("ubs_fp32_probe_workspace_bytes"), dev)
    flops = ctypes.c_double(0)
    best = 0.0
    for it in (2000, 2000, 2000):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        L.call("ubs_fp32_probe", it, L.ptr(ws), ws.numel(), ctypes.byref(flops), L.stream(dev))
        e1.record()
        e1.synchronize()
        best = max(best, flops.value / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    return best


def mufu_peak(dev):
    """XU issue rate (T MUFU ops/s) from the library's probe, best of three."""
    from ubs import _lib as L
    import ctypes
    ws = L.workspace(L.query("ubs_fp32_probe_workspace_bytes"), dev)
    ops = ctypes.c_double(0)
    best = 0.0
    for it in (500, 500, 500):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        L.call("ubs_mufu_probe", it, L.ptr(ws), ws.numel(), ctypes.byref(ops), L.stream(dev))
        e1.record()
        e1.synchronize()
        best = max(best, ops.value / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    return best


def count_pairs(p, cam, ri, rj, bg, dev):
    """(contributing pairs, intersections, visible primitives, evaluated
    forward pairs, backward pairs) of one forward (device counters)."""
    import ctypes
    from gsplat.cuda import _wrapper as Wr
    from ubs import _lib as L
    from ubs import scene as S
    with torch.no_grad():
        _, _, meta = S.render_view(p, cam, bg, ri, rj, tile_size=TILE)
        m2, cn = meta["means2d"], meta["conics"]
        op, be = meta["opacities"].contiguous(), meta["betas"].contiguous()
        fl, offs = meta["flatten_ids"], meta["isect_offsets"]
        C, N = op.shape
        T = fl.numel()
        colors = p["rgb"].detach().expand(1, -1, -1).contiguous()
        ws = L.workspace(L.query("ubs_raster_workspace_bytes", T, 3), dev)
        oc = torch.empty(1, HEIGHT, WIDTH, 3, device=dev)
        oa = torch.empty(1, HEIGHT, WIDTH, 1, device=dev)
        li = torch.empty(1, HEIGHT, WIDTH, dtype=torch.int32, device=dev)
        st = L.stream(dev)
        L.call("ubs_raster_pack", C, N, 3, T, L.ptr(fl), L.ptr(m2), L.ptr(cn), L.ptr(op),
               L.ptr(be), L.ptr(colors), L.ptr(ws), ws.numel(), st)
        L.call("ubs_raster_fwd_packed", C, N, 3, T, L.ptr(colors), L.ptr(bg.view(1, 3)), None,
               WIDTH, HEIGHT, TILE, meta["tile_width"], meta["tile_height"], L.ptr(offs),
               L.ptr(oc), L.ptr(oa), L.ptr(li), 1, L.ptr(ws), ws.numel(), st)
        counts = (ctypes.c_uint64 * 3)()
        L.call("ubs_raster_pair_counts", L.ptr(ws), ctypes.cast(counts, ctypes.c_void_p), st)
        del Wr
        return (int(counts[0]), int(T), int((meta["radii"] > 0).sum()), int(counts[1]),
                int(counts[2]))


def read_profile_traffic(kernel):
    """DRAM bytes per launch from a committed ncu summary (profiles/), if any."""
    path = os.path.join(ROOT, "profiles", kernel + "_1M_1080p.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


# --------------------------------------------- batched and served configs
def _ref_pipeline():
    try:
        import ref_gpu as RG
        return RG.RefPipeline() if RG.available() else None
    except Exception:  # noqa: BLE001
        return None


class TrainViews:
    """Fused forward + L1 + backward over all views in one launch."""

    def __init__(self, p, cams, dev, tile):
        from ubs.render import Renderer, Views
        self.p = p
        self.r = Renderer(dim=p["scale"].shape[1], tile_size=tile)
        self.views = Views(cams, tile_size=tile, device=dev)
        g = torch.Generator().manual_seed(3)
        self.target = torch.rand(self.views.n_pixels, 3, generator=g).to(dev)
        self.bg = torch.zeros(len(cams), 3, device=dev)
        with torch.no_grad():
            self.r.render(p, self.views, self.bg, check=True)

    def step(self):
        for v in self.p.values():
            v.grad = None
        colors, _ = self.r.render(self.p, self.views, self.bg, check=False)
        l1_loss(colors, self.target).backward()


def _train_views(p, cams, dev, tile, reps, flush):
    """ms per fused step (after two warm-up steps) and the intersection count."""
    tv = TrainViews(p, cams, dev, tile)
    for _ in range(2):
        tv.step()
    ms = time_steps(tv.step, reps, dev, flush)
    tv.r._check_pending()
    return ms, tv.r.last_isects


def _ref_train_views(rp, p, cams, dev, reps, flush):
    """ms per step of the reference's kernels, one view per launch."""
    ri, rj = None, None
    from ubs import scene as S
    ri, rj = S.rest_indices(p["scale"].shape[1], dev)
    g = torch.Generator().manual_seed(3)
    targets = [torch.rand(3, c.height, c.width, generator=g).to(dev) for c in cams]
    bg = torch.zeros(3, device=dev)

    def step():
        for v in p.values():
            v.grad = None
        for c, t in zip(cams, targets):
            img, _, _ = rp.render_view(p, c.viewmat, c.K, c.width, c.height, c.center, bg, ri, rj,
                                       tile_size=TILE, timestamp=c.timestamp)
            ((img - t).abs().mean() / len(cams)).backward()

    step()
    return time_steps(step, reps, dev, flush)


def look_at_camera(eye, width, height, focal):
    """Camera at `eye` looking at the origin, up +y, OpenCV axes, principal
    point at the image centre."""
    from ubs import scene as S
    e = torch.tensor(eye, dtype=torch.float64)
    f = -e / e.norm()
    r = torch.linalg.cross(f, torch.tensor([0.0, 1.0, 0.0], dtype=torch.float64))
    r = r / r.norm()
    u = torch.linalg.cross(r, f)
    Rw = torch.stack([r, -u, f], 0)
    vm = torch.eye(4, dtype=torch.float64)
    vm[:3, :3] = Rw
    vm[:3, 3] = -Rw @ e
    K = torch.tensor([[focal, 0.0, width / 2], [0.0, focal, height / 2], [0.0, 0.0, 1.0]])
    return S.Camera(vm.float(), K, width, height)


def run_config_a(dev, flush):
    """The reference's CPU-runnable case: 10k 6-D primitives (xyz in
    [-1, 1]^3), 256x256, fx = fy = 300, camera at (0, 0, -3) looking at the
    origin, L1 loss: forward and forward + backward through the oracle port
    on the host cores (all threads, then one thread) -- a reported baseline
    -- and through the fused GPU path on the same scene."""
    import oracle as orc
    from ubs.render import Renderer, Views
    W = H = 256
    cam = look_at_camera((0.0, 0.0, -3.0), W, H, 300.0)
    cs = CpuSample(10_000, 0, width=W, height=H, cam=cam, xyz_range=1.0)

    def cpu_times(reps=3):
        fwd = min(cs.forward() for _ in range(reps))
        step = min(cs.step(1, 0, 1) for _ in range(reps))
        return {"fwd_ms": fwd * 1e3, "fwd_bwd_ms": step * 1e3}

    threads = orc.num_threads()
    cpu_all = cpu_times()
    orc.set_threads(1)
    try:
        cpu_one = cpu_times()
    finally:
        orc.set_threads(threads)
    p = {k: torch.from_numpy(v).to(dev).contiguous() for k, v in cs.p.items()}
    p = {k: torch.nn.Parameter(v) for k, v in p.items()}
    cam_d = type(cam)(cam.viewmat.to(dev), cam.K.to(dev), W, H)
    views = Views([cam_d], tile_size=TILE, device=dev)
    r = Renderer(dim=DIM, tile_size=TILE)
    target = torch.from_numpy(cs.target_hwc).to(dev).reshape(-1, 3).contiguous()
    with torch.no_grad():
        r.render(p, views, None, check=True)

    def g_fwd():
        with torch.no_grad():
            r.render(p, views, None, check=False)

    def g_step():
        for v in p.values():
            v.grad = None
        colors, _ = r.render(p, views, None, check=False)
        l1_loss(colors, target).backward()

    for _ in range(3):
        g_step()
    fwd_ms = time_steps(g_fwd, 50, dev, flush)
    step_ms = time_steps(g_step, 50, dev, flush)
    r._check_pending()
    return {"workload": "10k 6-D primitives, 256x256 (fx=fy=300), camera at (0, 0, -3) looking "
                        "at the origin, forward + L1 loss + backward",
            "gpu": {"fwd_ms": fwd_ms, "fwd_bwd_ms": step_ms,
                    "path": "fused scene render, kernel by kernel"},
            "cpu": dict(cpu_all, threads=threads, kind="port",
                        what="the oracle port (C++ restatement, OpenMP) on the host cores, a "
                             "reported baseline"),
            "cpu_1_thread": dict(cpu_one, threads=1),
            "intersections": cs.n_isects}


def config_views(name, dev):
    """Parameters and cameras of config C (500k 7-D, 8 timestamped views
    1352x1014) or D (3M 6-D, 4 views of mixed resolution)."""
    from ubs import scene as S
    if name == "C":
        p = S.synthetic_params(500_000, 7, seed=0, xyz_range=2.0, device=dev)
        rng = np.random.default_rng(0)
        cams = [S.orbit_view(100 + i, 4.0, 1352, 1014, 1056.25, 1056.25,
                             timestamp=float(rng.uniform()), device=dev) for i in range(8)]
    else:
        p = S.synthetic_params(3_000_000, 6, seed=0, xyz_range=2.0, device=dev)
        res = [(1920, 1080), (1600, 1064), (1280, 720), (960, 540)]
        cams = [S.orbit_view(200 + i, 4.0, w, h, 1500.0 * w / 1920, 1500.0 * w / 1920, device=dev)
                for i, (w, h) in enumerate(res)]
    for v in p.values():
        v.requires_grad_(True)
    return p, cams


def profile_config(name, dev, warmup):
    """The batched step of config C or D, warmup + 1 times, for an ncu capture."""
    p, cams = config_views(name, dev)
    st = TrainViews(p, cams, dev, TILE)
    for _ in range(warmup + 1):
        st.step()
    torch.cuda.synchronize()
    st.r._check_pending()
    print("profile run: config %s" % name, flush=True)


def run_config_c(dev, flush, rp):
    """500k 7-D dynamic primitives, 8 views of 1352x1014 with timestamps, one
    batched forward + backward."""
    p, cams = config_views("C", dev)
    ms, isects = _train_views(p, cams, dev, TILE, 10, flush)
    out = {"workload": "500k 7-D primitives, 8 views 1352x1014 (fx=fy=1056.25) with timestamps "
                       "U[0,1], one fused forward + L1 + backward", "ms_per_step": ms,
           "it_per_s": 1000.0 / ms, "views_per_s": 8000.0 / ms, "isects": isects}
    if rp is not None:
        r_ms = _ref_train_views(rp, p, cams, dev, 3, flush)
        out["ref_gpu_plain"] = {"ms_per_step": r_ms, "it_per_s": 1000.0 / r_ms,
                                "what": "reference kernels, one view per launch"}
    return out


def run_config_d(dev, flush, rp):
    """3M 6-D primitives, 4 views of mixed resolution in one launch, tile size
    picked by the autotuner, peak memory reported."""
    from ubs.autotune import TileAutotuner
    p, cams = config_views("D", dev)
    tuner = TileAutotuner(reps=3)
    states = {}

    def tune_step(ts):
        if ts not in states:
            states[ts] = TrainViews(p, cams, dev, ts)
        states[ts].step()

    best = tuner.pick("configD", tune_step)
    for st in states.values():
        st.r._check_pending()
    states.clear()
    torch.cuda.synchronize()
    torch.cuda.reset_peak_memory_stats(dev)
    ms, isects = _train_views(p, cams, dev, best, 10, flush)
    peak = torch.cuda.max_memory_allocated(dev)
    out = {"workload": "3M 6-D primitives, views 1920x1080 + 1600x1064 + 1280x720 + 960x540 "
                       "(fx = 1500 W/1920) in one fused forward + L1 + backward",
           "tile_size": best, "blend_variant": {"forward": tuner.choice("configD")[1],
                                                "backward": tuner.choice("configD")[2]},
           "autotune_ms": {"tile %d / fwd variant %d / bwd variant %d" % k: round(v, 3)
                           for k, v in tuner.timings("configD").items()},
           "ms_per_step": ms, "it_per_s": 1000.0 / ms, "isects": isects,
           "peak_memory_bytes": int(peak),
           "peak_memory_note": "torch.cuda.max_memory_allocated over the timed steps "
                               "(parameters, gradients, workspaces, images)"}
    from ubs.autotune import set_blend_variant
    set_blend_variant(0, 0)  # the later measurements use the default variant
    if rp is not None:
        r_ms = _ref_train_views(rp, p, cams, dev, 3, flush)
        out["ref_gpu_plain"] = {"ms_per_step": r_ms, "it_per_s": 1000.0 / r_ms,
                                "what": "reference kernels, one view per launch"}
    return out


SLO_MS = 10.0
SERVED_RATES = (200, 300, 400, 450, 500, 550, 600, 650, 700, 800, 1000)
PLAIN_RATES = (25, 50, 100, 150, 200, 300)


def slo_sweep(run_at, rates, slo_ms=SLO_MS):
    """Latency/throughput at each Poisson arrival rate; `best` is the rate
    with the most frames/s among those whose p99 latency stays under slo_ms."""
    rows = []
    for rate in rates:
        st = run_at(rate)
        st["rate"] = rate
        rows.append(st)
    ok = [r for r in rows if r["p99_ms"] < slo_ms]
    best = max(ok, key=lambda r: r["frames_per_s"]) if ok else None
    return {"slo_p99_ms": slo_ms, "rates": rows,
            "best": None if best is None else {k: best[k] for k in
                                               ("rate", "frames_per_s", "p50_ms", "p99_ms",
                                                "mean_batch")}}


def run_serving(dev, rp, duration=3.0, rate=200.0, sweep_s=1.5):
    """Resident scenes of 500k, 1M and 3M 6-D primitives; Poisson requests at
    `rate`/s with resolutions uniform over 640x480, 1280x720, 1920x1080; then
    a sweep of arrival rates per form for the highest throughput whose p99
    latency stays under 10 ms."""
    from ubs import scene as S
    from ubs.serve import ServeConfig, Server, latency_stats, poisson_trace, run_plain
    sizes = {"s500k": 500_000, "s1m": 1_000_000, "s3m": 3_000_000}
    scenes = {k: S.synthetic_params(n, 6, seed=i, xyz_range=2.0, device=dev)
              for i, (k, n) in enumerate(sizes.items())}
    res = [(640, 480), (1280, 720), (1920, 1080)]
    # a batch's estimated intersections are bounded so that one batch's device
    # time stays a fraction of the latency target
    cfg = ServeConfig(max_slots=4, max_batch_views=8, max_batch_isects=6_000_000)
    srv = Server(scenes, cfg)
    srv.calibrate({k: S.orbit_view(7, 4.0, 1280, 720, 1000.0, 1000.0, device=dev) for k in scenes})
    trace = poisson_trace(rate, duration, list(scenes), res, seed=0, device=dev)
    srv.run(trace[:40], realtime=False)  # warm-up (allocator, kernels)
    served = latency_stats(srv.run(trace, realtime=True))
    sat_done = srv.run(trace, realtime=False)
    saturated = latency_stats(sat_done)
    out = {"workload": "resident scenes of 500k, 1M, 3M 6-D primitives; Poisson arrivals at "
                       "%g req/s for %g s (%d requests), resolutions uniform over 640x480, "
                       "1280x720, 1920x1080, random radius-4 orbit cameras; latency = arrival "
                       "to image in pinned host memory" % (rate, duration, len(trace)),
           "served": served, "served_saturated": saturated, "reruns": srv.reruns,
           "max_batch_isects": cfg.max_batch_isects}
    bg = torch.zeros(3, device=dev)
    ri, rj = S.rest_indices(6, dev)

    def trace_at(r):
        return poisson_trace(r, sweep_s, list(scenes), res, seed=int(r), device=dev)

    def dropin_one(r):
        with torch.no_grad():
            img, _, _ = S.render_view(scenes[r.scene], r.camera, bg, ri, rj, tile_size=TILE)
        return img

    run_plain(dropin_one, trace[:20], realtime=False)
    out["plain_dropin"] = latency_stats(run_plain(dropin_one, trace, realtime=True))
    out["plain_dropin_saturated"] = latency_stats(run_plain(dropin_one, trace, realtime=False))
    sweeps = {"served": slo_sweep(lambda r: latency_stats(srv.run(trace_at(r), realtime=True)),
                                  SERVED_RATES),
              "plain_dropin": slo_sweep(
                  lambda r: latency_stats(run_plain(dropin_one, trace_at(r), realtime=True)),
                  PLAIN_RATES)}
    if rp is not None:
        def ref_one(r):
            c = r.camera
            with torch.no_grad():
                img, _, _ = rp.render_view(scenes[r.scene], c.viewmat, c.K, c.width, c.height,
                                           c.center, bg, ri, rj, tile_size=TILE)
            return img

        run_plain(ref_one, trace[:20], realtime=False)
        out["plain_ref_gpu"] = latency_stats(run_plain(ref_one, trace, realtime=True))
        out["plain_ref_gpu_saturated"] = latency_stats(run_plain(ref_one, trace,
                                                                 realtime=False))
        sweeps["plain_ref_gpu"] = slo_sweep(
            lambda r: latency_stats(run_plain(ref_one, trace_at(r), realtime=True)), PLAIN_RATES)
    out["slo_sweep"] = sweeps
    # the target: served frames/s under the latency bound over the plain
    # one-request-per-launch form's, at its own best rate under the same bound
    # and at its saturated (unbounded-latency) throughput
    sb = sweeps["served"]["best"]
    summary = {"served_fps_at_slo": sb and sb["frames_per_s"], "served_rate_at_slo": sb and sb["rate"]}
    for form, sat in (("plain_dropin", "plain_dropin_saturated"),
                      ("plain_ref_gpu", "plain_ref_gpu_saturated")):
        if form not in sweeps:
            continue
        pb = sweeps[form]["best"]
        summary[form] = {
            "fps_at_slo": pb and pb["frames_per_s"], "rate_at_slo": pb and pb["rate"],
            "saturated_fps": out[sat]["frames_per_s"],
            "ratio_at_slo": (sb["frames_per_s"] / pb["frames_per_s"]) if (sb and pb) else None,
            "ratio_vs_saturated": (sb["frames_per_s"] / out[sat]["frames_per_s"]) if sb else None}
    out["slo_summary"] = summary
    return out


# ------------------------------------------------------- CPU (oracle port)
def cpu_problem(n_prims, seed, width=WIDTH, height=HEIGHT, cam=None, xyz_range=2.0):
    from ubs import scene as S
    p = {k: v.numpy().astype(np.float32) for k, v in
         S.synthetic_params(n_prims, DIM, seed=seed, xyz_range=xyz_range, device="cpu").items()}
    if cam is None:
        cam = S.orbit_view(seed, 4.0, width, height, FOCAL, FOCAL, device="cpu")
    target = torch.rand(3, height, width, generator=torch.Generator().manual_seed(seed + 7)).numpy()
    ri, rj = S.rest_indices(DIM)
    return p, cam, ri.numpy(), rj.numpy(), target


class CpuSample:
    """The training step of the headline workload on the host CPU through the
    oracle port (C++ with OpenMP; the reference has no CPU blend), timed as a
    bounded sample: step k runs the per-primitive forward, intersection sort
    and per-primitive backward on the k-th of FP equal slices of the
    primitives, and the blend forward + backward (with the L1 loss gradient)
    on the tile rows ty % F == k % F (the blend's inputs for those rows come
    from one full untimed forward at set-up; its buffers are reused, and the
    sampled gradients are not reset between steps since only the time is
    used).  Each part's time is scaled to the whole frame (x N / slice,
    x rows / sampled rows); consecutive steps cycle over slices and rows."""

    def __init__(self, n_prims, seed=0, width=WIDTH, height=HEIGHT, cam=None, xyz_range=2.0):
        import oracle as orc
        self.orc = orc
        self.W, self.H = width, height
        self.p, self.cam, self.ri, self.rj, self.target = cpu_problem(n_prims, seed, width,
                                                                       height, cam, xyz_range)
        self.N = n_prims
        self.tw, self.th = math.ceil(width / TILE), math.ceil(height / TILE)
        t0 = time.perf_counter()
        self.full = self._prim_forward(slice(None))
        _, ids, self.fl = orc.isect_tiles(self.full["m2"], self.full["radii"], self.full["d"],
                                          TILE, self.tw, self.th)
        self.n_isects = len(ids)
        self.offs = orc.isect_offset_encode(ids, 1, self.tw, self.th)
        self.t_prim_fwd_full = time.perf_counter() - t0
        # reused blend buffers: a sampled step writes only its rows, so that
        # no full-frame allocation or loss is scaled with the sample
        C = 1
        self.out_f = (np.zeros((C, height, width, 3), np.float32),
                      np.zeros((C, height, width, 1), np.float32),
                      np.zeros((C, height, width), np.int32))
        self.out_b = (np.zeros((C, n_prims, 2), np.float32), np.zeros((C, n_prims, 3), np.float32),
                      np.zeros((C, n_prims, 3), np.float32), np.zeros((C, n_prims), np.float32),
                      np.zeros((C, n_prims), np.float32))
        self.v_oc = np.zeros((C, height, width, 3), np.float32)
        self.v_oa = np.zeros((C, height, width, 1), np.float32)
        self.target_hwc = np.ascontiguousarray(self.target.transpose(1, 2, 0))

    def _prim_forward(self, sl):
        orc, p = self.orc, self.p
        f32 = np.float32
        scale, ltri = p["scale"][sl], p["l_triangle"][sl]
        sp = (np.log1p(np.exp(-np.abs(scale))) + np.maximum(scale, 0)).astype(f32)
        beta = (4.0 * np.exp(p["beta"][sl])).astype(f32)
        opac = (1.0 / (1.0 + np.exp(-p["opacity"][sl]))).astype(f32)
        vm = self.cam.viewmat.numpy()[None].astype(f32)
        K = self.cam.K.numpy()[None].astype(f32)
        center = self.cam.center.numpy().astype(f32)
        vd = p["xyz"][sl] - center[None]
        q = (vd / np.linalg.norm(vd, axis=-1, keepdims=True)).astype(f32)
        R = orc.l_triangle_to_rotmat(ltri)
        cov = orc.rot_scale_l_triangle_to_covar(R, sp, ltri, self.ri, self.rj)
        m_nd = np.concatenate([p["xyz"][sl], p["mean"][sl]], 1)
        om, oV, oo = orc.cond_mean_convariance_opacity(m_nd, cov, opac, beta[:, 1:], q)
        c6 = np.ascontiguousarray(oV[:, [0, 0, 0, 1, 1, 2], [0, 1, 2, 1, 2, 2]])
        radii, m2, d, cn, _ = orc.fully_fused_projection(om, c6, None, None, vm, K, self.W,
                                                         self.H)
        return dict(sp=sp, beta=beta, opac=opac, vm=vm, K=K, q=q, R=R, cov=cov, m_nd=m_nd,
                    om=om, oV=oV, oo=oo, c6=c6, radii=radii, m2=m2, d=d, cn=cn, ltri=ltri)

    def _prim_backward(self, f, vm2, vcn, vo):
        orc = self.orc
        vmeans, vc6, _, _, _ = orc.fully_fused_projection_bwd(
            f["om"], f["c6"], None, None, f["vm"], f["K"], self.W, self.H, 0.3, f["radii"],
            f["cn"], None, vm2, None, vcn)
        v_oV = np.zeros_like(f["oV"])
        for k, (i, j) in enumerate(zip([0, 0, 0, 1, 1, 2], [0, 1, 2, 1, 2, 2])):
            v_oV[:, i, j] = vc6[:, k]
        gm, gV, go, gb = orc.cond_mean_convariance_opacity_bwd(
            f["m_nd"], f["cov"], f["opac"], f["beta"][:, 1:], f["q"], vmeans, v_oV,
            vo.reshape(-1, 1))
        vr, vs, vl = orc.rot_scale_l_triangle_to_covar_bwd(f["R"], f["sp"], f["ltri"], self.ri,
                                                           self.rj, gV)
        vl[:, :3] += orc.l_triangle_to_rotmat_bwd(vr)
        return gm, vs, vl

    def forward(self):
        """Seconds of one full forward: per-primitive forward, intersection
        sort and offsets, blend."""
        orc = self.orc
        t0 = time.perf_counter()
        f = self._prim_forward(slice(None))
        _, ids, fl = orc.isect_tiles(f["m2"], f["radii"], f["d"], TILE, self.tw, self.th)
        offs = orc.isect_offset_encode(ids, 1, self.tw, self.th)
        orc.rasterize_to_pixels(f["m2"], f["cn"], self.p["rgb"][None], f["oo"].reshape(1, -1),
                                f["beta"][:, 0].reshape(1, -1), self.W, self.H, TILE, offs, fl,
                                backgrounds=np.zeros((1, 3), np.float32))
        return time.perf_counter() - t0

    def step(self, F, k, FP=None):
        """Scaled seconds of one full-frame step, sampled as described above
        (primitive slices of 1/FP, default F)."""
        orc, full = self.orc, self.full
        FP = FP or F
        lo, hi = k % FP * self.N // FP, (k % FP + 1) * self.N // FP
        sl = slice(lo, hi)
        t0 = time.perf_counter()
        f = self._prim_forward(sl)
        orc.isect_tiles(f["m2"], f["radii"], f["d"], TILE, self.tw, self.th)
        t_prim = time.perf_counter() - t0
        t1 = time.perf_counter()
        colors = self.p["rgb"][None]
        op, be = full["oo"].reshape(1, -1), full["beta"][:, 0].reshape(1, -1)
        bg = np.zeros((1, 3), np.float32)
        off = k % F
        oc, oa, li = orc.rasterize_to_pixels(full["m2"], full["cn"], colors, op, be, self.W,
                                             self.H, TILE, self.offs, self.fl, backgrounds=bg,
                                             row_step=F, row_offset=off, out=self.out_f)
        # L1 loss gradient on the sampled pixel rows
        for ty in range(off, self.th, F):
            r0, r1 = ty * TILE, min(self.H, (ty + 1) * TILE)
            d = oc[0, r0:r1] - self.target_hwc[r0:r1]
            self.v_oc[0, r0:r1] = np.sign(d) / (3.0 * self.H * self.W)
        vm2, vcn, _, vo, _ = orc.rasterize_to_pixels_bwd(
            full["m2"], full["cn"], colors, op, be, self.W, self.H, TILE, self.offs, self.fl, oa,
            li, self.v_oc, self.v_oa, backgrounds=bg, row_step=F, row_offset=off,
            out=self.out_b)
        t_blend = time.perf_counter() - t1
        t2 = time.perf_counter()
        self._prim_backward(f, vm2[:, sl], vcn[:, sl], vo[:, sl])
        t_prim += time.perf_counter() - t2
        rows = len(range(off, self.th, F))
        return t_prim * self.N / (hi - lo) + t_blend * self.th / max(1, rows)


CPU_BUDGET_S = 120.0  # wall time the timed CPU steps may take


def run_cpu(steps, warmup, n_prims):
    """Bounded CPU sample of the training step: F (a power of two) is the
    smallest row sampling that keeps steps + warmup sampled steps within about
    CPU_BUDGET_S seconds; primitives are sliced at most 8 ways (finer slices
    would scale the stages' fixed per-call costs up with them)."""
    import oracle as orc
    cs = CpuSample(n_prims, 0)
    # a full step is ~2.2x the per-primitive forward plus the blend; estimate
    # the blend from one 1/16 row sample (untimed)
    t_est = cs.step(16, 0)
    F = 1
    while F < 64 and (t_est / F) * (steps + warmup) > CPU_BUDGET_S:
        F *= 2
    FP = min(F, 8)
    for i in range(warmup):
        cs.step(F, i, FP)
    total = 0.0
    for i in range(steps):
        total += cs.step(F, warmup + i, FP)
    dt = total / steps
    return {"value": 1.0 / dt, "unit": "it/s", "ms_per_step": dt * 1e3,
            "cores": orc.num_threads(), "kind": "port",
            "sample": "per step: per-primitive forward, intersection sort and backward on 1/%d "
                      "of the %d primitives and the blend forward + backward on every %dth of "
                      "the %d tile rows (cycling slices and rows), each scaled to the full "
                      "1920x1080 frame (C++ oracle port, OpenMP)" % (FP, n_prims, F, cs.th)}


def headline_summary(value, e2e_val, render_fps, d_ms, d_fwd_ms, ref_gpu, roofline, configs):
    """The figures a reader compares, in one short dict: train it/s (graph
    replay, end to end), render FPS, the drop-in operators' and the
    reference kernels' plain form on the same GPU, the blend roofline
    fractions, and configs C, D and E against the reference's plain form."""
    def r3(x):
        return None if x is None else round(float(x), 3)
    out = {"train_it_s": r3(value), "e2e_it_s": r3(e2e_val), "render_fps": r3(render_fps),
           "dropin_it_s": r3(1000.0 / d_ms), "dropin_render_fps": r3(1000.0 / d_fwd_ms)}
    if ref_gpu and "value" in ref_gpu:
        out["ref_gpu_it_s"] = r3(ref_gpu["value"])
        out["ref_gpu_render_fps"] = r3(ref_gpu["render_fps"])
        out["train_vs_ref_gpu"] = r3(value / ref_gpu["value"])
        out["render_vs_ref_gpu"] = r3(render_fps / ref_gpu["render_fps"])
    out["roofline"] = {"kernel": roofline["kernel"], "fp32_frac": r3(roofline["frac"]),
                       "mufu_frac": r3(roofline["mufu"]["frac"]),
                       "launch_ms": r3(roofline["launch_ms"])}
    for name in ("C", "D"):
        c = (configs or {}).get(name) or {}
        if "ms_per_step" in c:
            e = {"ms_per_step": r3(c["ms_per_step"])}
            rg = c.get("ref_gpu_plain")
            if rg:
                e["ref_gpu_ms"] = r3(rg["ms_per_step"])
                e["vs_ref_gpu"] = r3(rg["ms_per_step"] / c["ms_per_step"])
            out["config_" + name] = e
    e = (configs or {}).get("E") or {}
    if "slo_summary" in e:
        out["serving_p99_slo"] = e["slo_summary"]
    return out


# ------------------------------------------------------------------- main
def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")

    if args.impl == "reference":
        # CPU reference arm: rank 0 only
        if rank == 0:
            steps, warmup = args.steps, args.warmup
            # each step is a bounded sample; keep the whole run within minutes
            r = run_cpu(steps, warmup, args.n_prims)
            line = {"metric": METRIC, "value": r["value"], "unit": "it/s", "impl": "reference",
                    "n_gpus": args.gpus, "steps": steps, "warmup": warmup,
                    "ms_per_step": r["ms_per_step"], "higher_is_better": True,
                    "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                    "data": "synthetic (seeded, benchmark distributions)",
                    "config": {"workload": WORKLOAD, "n_prims": args.n_prims, "dim": DIM,
                               "width": WIDTH, "height": HEIGHT, "tile_size": TILE,
                               "parallelism": "host CPU, %d threads" % r["cores"],
                               "l2": "n/a (host CPU; each step a bounded sample)",
                               "path": "C++ restatement of the reference's path (oracle), "
                                       "OpenMP over tiles and primitives"},
                    "cpu_baseline": {k: r[k] for k in ("value", "unit", "cores", "kind", "sample")},
                    "e2e": {"value": r["value"], "unit": "it/s", "h2d_bytes_per_step": 0,
                            "d2h_bytes_per_step": 0}}
            print(json.dumps(line), flush=True)
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
            dist.destroy_process_group()
        return

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    from ubs import _lib as L
    L.lib()
    if args.profile_config:
        profile_config(args.profile_config, dev, args.warmup)
        return
    p, cam, ri, rj, bg, target = make_problem(args.n_prims, rank, dev)
    fz = FusedStep(p, cam, bg, target, dev)
    if args.profile_neighbours:
        profile_neighbours(p, cam, dev)
        return
    if args.profile and args.dropin:
        for _ in range(args.warmup + 1):
            gpu_step(p, cam, ri, rj, bg, target)
        torch.cuda.synchronize()
        print("profile run (drop-in operators)", flush=True)
        return
    if args.profile and args.eager:
        fz.prime()
        for _ in range(args.warmup + 1):
            fz.step()
        torch.cuda.synchronize()
        fz.renderer._check_pending()
        print("profile run: %d intersections" % fz.renderer.last_isects, flush=True)
        return
    from ubs.render import GraphedStep, Renderer
    g_target = fz.target.clone()
    g_ren = Renderer(dim=DIM, tile_size=TILE)
    prof_slots = 64 * 4
    gs = GraphedStep(g_ren, p, fz.views, fz.bg,
                     lambda colors, alphas: l1_loss(colors, g_target),
                     before_capture=lambda: L.profile_start(prof_slots))
    if args.profile:
        L.profile_stop()
        for _ in range(args.warmup + 1):
            gs.replay()
        torch.cuda.synchronize()
        gs.check()
        print("profile run (graph): %d intersections" % g_ren.last_isects, flush=True)
        return
    flush = l2_flush_buffer(dev)
    clocks = ClockSampler()
    clocks.start()
    for _ in range(max(3, args.warmup)):
        gs.replay()
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    clocks.mark("t0")
    t_wall = time.perf_counter()
    ms = time_steps(gs.replay, args.steps, dev, flush, after=L.profile_sample)
    kernels = L.profile_stop()
    wall = time.perf_counter() - t_wall
    clocks.mark("t1")
    gs.check()  # raises if the replayed frame overflowed its buffers
    # kernel launches of this library inside the timed region: the graph's
    # library kernels, once per replay (the host-side counter sees the capture)
    launches = gs.launches_per_replay * args.steps
    torch.cuda.synchronize()
    ms_max, value = replica_throughput(ms, world, dev)
    kernel_ms = {k: t / args.steps for k, (n, t) in kernels.items()}

    # end to end through the public API: parameters and target copied from
    # pinned host memory into the step's tensors every step, the loss read back
    host = {k: v.detach().cpu().pin_memory() for k, v in p.items()}
    host_target = g_target.cpu().pin_memory()
    h2d = sum(v.numel() * 4 for v in host.values()) + host_target.numel() * 4
    loss_host = torch.empty(1, pin_memory=True)

    def e2e_step():
        with torch.no_grad():
            for k, v in p.items():
                v.copy_(host[k], non_blocking=True)
            g_target.copy_(host_target, non_blocking=True)
        loss = gs.replay()
        loss_host.copy_(loss.detach().view(1), non_blocking=True)

    for _ in range(2):
        e2e_step()
    e2e_serial_ms = time_steps(e2e_step, args.steps, dev, flush)
    gs.check()
    _, e2e_serial = replica_throughput(e2e_serial_ms, world, dev)

    # the same, double-buffered through ubs.render.HostFedStep: step k+1's
    # host-to-device copies run on a copy stream during step k's compute; the
    # timed region spans K consecutive steps (every copy and loss read inside
    # it; each step's 165 MB of fresh inputs exceeds the 129 MB L2)
    from ubs.render import HostFedStep

    def make_inputs():
        q = {k: torch.nn.Parameter(v.detach().clone()) for k, v in p.items()}
        t = g_target.clone()
        return q, [q[k] for k in p] + [t], lambda c, a: l1_loss(c, t)

    hf = HostFedStep(Renderer(dim=DIM, tile_size=TILE), fz.views, fz.bg, make_inputs)
    feed_host = [host[k] for k in p] + [host_target]
    for _ in range(4):
        hf.step(feed_host)
    hf.losses()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    hf.start()
    for _ in range(args.steps):
        hf.step(feed_host)
        if len(hf.pending) >= hf.ring - 1:
            hf.losses()
    e1.record()
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    e2e_losses = hf.losses()
    hf.check()
    _, e2e_val = replica_throughput(e2e_ms, world, dev)
    del hf
    clocks.stop()
    # the same step without the graph (one launch per kernel from the host)
    fz.prime()
    for _ in range(3):
        fz.step()
    eager_ms = time_steps(fz.step, max(20, min(args.steps, 100)), dev, flush)
    fz.renderer._check_pending()
    fwd_ms = time_steps(fz.forward, max(5, min(args.steps, 20)), dev, flush)
    fz.renderer._check_pending()

    K2 = max(5, min(args.steps, 20))
    # a full training iteration: the step plus the Adam update of the seven
    # parameter groups, on a copy of the parameters (they change every step)
    train_iter = None
    try:
        from ubs.loss import l1_ssim_loss
        from ubs.optim import FusedAdam
        from ubs.render import GraphedStep as _GS, Renderer as _R
        p2 = {k: torch.nn.Parameter(v.detach().clone()) for k, v in p.items()}
        groups2 = [{"params": [p2[k]], "lr": lr, "name": k} for k, lr in TRAIN_LRS.items()]
        g_t2 = fz.target.clone().view(1, HEIGHT, WIDTH, 3)
        gs2 = _GS(_R(dim=DIM, tile_size=TILE), p2, fz.views, fz.bg,
                  lambda c, a: l1_ssim_loss(c.view(1, HEIGHT, WIDTH, 3), g_t2, LAMBDA_DSSIM,
                                            channels_last=True),
                  optimizer=FusedAdam(groups2, lr=0.0, eps=1e-15))
        for _ in range(3):
            gs2.replay()
        it_ms = time_steps(gs2.replay, K2, dev, flush)
        gs2.check()
        # the Adam launch alone (eager, the same optimizer and gradients)
        L.profile_start(64)
        for _ in range(10):
            flush.fill_(2.0)
            gs2.optimizer.step()
        torch.cuda.synchronize()
        adam_prof = L.profile_stop()
        n_ad, t_ad = adam_prof.get("adam", (0, 0.0))
        adam_ms = t_ad / max(1, n_ad)
        adam_bytes = sum(v.numel() for v in p2.values()) * 28  # p, g, m, v read; p, m, v written
        adam_gbs = adam_bytes / (adam_ms * 1e-3) / 1e9 if adam_ms else None
        p3 = {k: torch.nn.Parameter(v.detach().clone()) for k, v in p.items()}
        groups3 = [{"params": [p3[k]], "lr": lr, "name": k} for k, lr in TRAIN_LRS.items()]
        adam3 = torch.optim.Adam(groups3, lr=0.0, eps=1e-15)
        fz3 = FusedStep(p3, cam, bg, target, dev, loss="l1_ssim_torch")
        fz3.prime()

        def torch_adam_iter():
            fz3.step()
            adam3.step()

        for _ in range(3):
            torch_adam_iter()
        it3_ms = time_steps(torch_adam_iter, K2, dev, flush)
        fz3.renderer._check_pending()
        hbm_peak = None
        try:
            hbm_peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs")
        except (OSError, ValueError):
            pass
        train_iter = {"value": 1000.0 / it_ms, "unit": "it/s", "ms_per_step": it_ms,
                      "adam": {"kernel_ms": adam_ms, "bytes": adam_bytes, "achieved_gbs": adam_gbs,
                               "frac_of_hbm": adam_gbs / hbm_peak if (adam_gbs and hbm_peak)
                               else None,
                               "what": "one FusedAdam launch over the 35 floats per primitive "
                                       "of the 7 groups, 28 B per element (HBM bound)"},
                      "what": "render + the reference's training loss 0.8 L1 + 0.2 (1 - SSIM) "
                              "(one fused loss kernel) + backward + Adam update of the 7 "
                              "parameter groups (FusedAdam, one kernel), as one CUDA graph",
                      "with_torch_adam": {"value": 1000.0 / it3_ms, "ms_per_step": it3_ms,
                                          "what": "the fused render launched kernel by kernel, "
                                                  "the loss with SSIM as utils/loss_utils.py "
                                                  "formulates it in PyTorch, then "
                                                  "torch.optim.Adam (the reference's "
                                                  "optimizer)"}}
        del gs2, p2, p3, fz3, adam3
    except Exception as e:  # noqa: BLE001
        train_iter = {"error": repr(e)[:300]}

    loss_res = None
    try:
        loss_res = bench_loss(dev, flush, max(10, min(args.steps, 50)))
    except Exception as e:  # noqa: BLE001
        loss_res = {"error": repr(e)[:300]}
    densify = None
    try:
        densify = bench_densify(p, dev)
    except Exception as e:  # noqa: BLE001
        densify = {"error": repr(e)[:300]}
    torch.cuda.empty_cache()
    scene_file = None
    try:
        scene_file = bench_scene_file(p, dev)
    except Exception as e:  # noqa: BLE001
        scene_file = {"error": repr(e)[:300]}
    viewer = None
    try:
        viewer = bench_viewer(p, cam, dev)
    except Exception as e:  # noqa: BLE001
        viewer = {"error": repr(e)[:300]}
    torch.cuda.empty_cache()

    # the drop-in operator sequence (gsplat.rendering.rasterization call path)
    d_step = lambda: gpu_step(p, cam, ri, rj, bg, target)  # noqa: E731
    for _ in range(3):
        d_step()
    L.profile_start(64 * (K2 + 1))
    d_ms = time_steps(d_step, K2, dev, flush)
    d_kernels = {k: round(t / K2, 4) for k, (n, t) in
                 sorted(L.profile_stop().items(), key=lambda x: -x[1][1])}

    def d_fwd():
        from ubs import scene as S
        with torch.no_grad():
            S.render_view(p, cam, bg, ri, rj, tile_size=TILE)
    d_fwd_ms = time_steps(d_fwd, K2, dev, flush)

    pairs, n_isects, n_visible, eval_pairs, bwd_pairs = count_pairs(p, cam, ri, rj, bg, dev)
    peak_fp32 = fp32_peak(dev)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak_mufu = mufu_peak(dev)
    dominant = max(kernel_ms, key=kernel_ms.get)
    n_dom, t_dom = kernels[dominant]
    dom_ms = t_dom / n_dom
    is_bwd = dominant == "raster_bwd"
    units = bwd_pairs if is_bwd else eval_pairs
    flop = units * PAIR_TEST_FLOP + pairs * (BWD_CONTRIB_FLOP if is_bwd else FWD_CONTRIB_FLOP)
    mufu = pairs * (BWD_CONTRIB_MUFU if is_bwd else FWD_CONTRIB_MUFU)
    fp32_ach = flop / (dom_ms * 1e-3) / 1e12
    mufu_ach = mufu / (dom_ms * 1e-3) / 1e12
    fp32_frac = fp32_ach / peak_fp32 if peak_fp32 else None
    mufu_frac = mufu_ach / peak_mufu if peak_mufu else None
    roofline = {
        "kernel": dominant, "bound": "fp32",
        "achieved": fp32_ach, "peak": peak_fp32, "unit": "TFLOP/s (FP32, FMA = 2 FLOPs)",
        "frac": fp32_frac,
        "traffic": read_profile_traffic(dominant),
        "algorithmic_work": "%d %s pairs x %d FLOPs + %d contributing pairs x %d FLOPs = %.2f "
                            "GFLOP per launch" % (
                                units, "backward (up to each pixel's last contributor)" if is_bwd
                                else "evaluated", PAIR_TEST_FLOP, pairs,
                                BWD_CONTRIB_FLOP if is_bwd else FWD_CONTRIB_FLOP, flop / 1e9),
        "mufu": {"ops_per_launch": mufu, "achieved": mufu_ach, "peak": peak_mufu,
                 "unit": "T MUFU ops/s", "frac": mufu_frac,
                 "peak_source": "XU probe kernel (exp2 chains) timed in this run"},
        "peak_source": "FP32 FMA probe kernel timed in this run (MEASURED_PEAKS.json has HBM "
                       "%s GB/s and bf16 only; the blend has no dense contraction)"
                       % peaks.get("hbm_gbs", "n/a"),
        "launch_ms": dom_ms,
        "timing": "CUDA events on the launching stream around each launch (graph event "
                  "nodes), every replay of the timed region",
    }

    # the reference's own kernels, plain one-view-per-launch path, same GPU
    ref_gpu = None
    if not args.no_ref_gpu and rank == 0:
        try:
            import ref_gpu as RG
            if RG.available():
                rp = RG.RefPipeline()

                def ref_step():
                    for v in p.values():
                        v.grad = None
                    img, _, _ = rp.render_view(p, cam.viewmat, cam.K, WIDTH, HEIGHT, cam.center,
                                               bg, ri, rj, tile_size=TILE)
                    (img - target).abs().mean().backward()

                def ref_fwd():
                    with torch.no_grad():
                        rp.render_view(p, cam.viewmat, cam.K, WIDTH, HEIGHT, cam.center, bg, ri,
                                       rj, tile_size=TILE)

                for _ in range(3):
                    ref_step()
                r_ms = time_steps(ref_step, K2, dev, flush)
                r_fwd_ms = time_steps(ref_fwd, K2, dev, flush)
                ref_gpu = {"value": 1000.0 / r_ms, "unit": "it/s", "ms_per_step": r_ms,
                           "render_fps": 1000.0 / r_fwd_ms,
                           "what": "the reference's CUDA kernels (built from its sources for "
                                   "sm_103) in its plain one-view-per-launch call sequence on "
                                   "this GPU; intersections sorted with torch.sort in place of "
                                   "its cub sort"}
        except Exception as e:  # noqa: BLE001
            ref_gpu = {"error": str(e)[:200]}

    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        try:
            r = run_cpu(1, 0, args.n_prims)
            cpu = {k: r[k] for k in ("value", "unit", "cores", "kind", "sample")}
        except Exception as e:  # noqa: BLE001
            cpu = {"error": str(e)[:200]}

    configs = None
    if not args.no_configs and rank == 0:
        rp = _ref_pipeline() if not args.no_ref_gpu else None
        configs = {}
        for name, fn in (("A", lambda: run_config_a(dev, flush)),
                         ("C", lambda: run_config_c(dev, flush, rp)),
                         ("D", lambda: run_config_d(dev, flush, rp)),
                         ("E", lambda: run_serving(dev, rp))):
            try:
                configs[name] = fn()
            except Exception as e:  # noqa: BLE001
                configs[name] = {"error": repr(e)[:300]}
            torch.cuda.empty_cache()

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "it/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded, benchmark distributions; reference datasets absent)",
            "config": {"workload": WORKLOAD, "n_prims": args.n_prims, "dim": DIM,
                       "width": WIDTH, "height": HEIGHT, "tile_size": TILE,
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "l2": "256 MB buffer written before every timed step (untimed); "
                             "per-step CUDA events",
                       "path": "fused scene render (ubs.render.Renderer), whole step "
                               "replayed as one CUDA graph (ubs.render.GraphedStep)"},
            "e2e": {"value": e2e_val, "unit": "it/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": 4, "ms_per_step": e2e_ms,
                    "how": "ubs.render.HostFedStep: parameters and target copied from pinned "
                           "host memory every step on a copy stream, double-buffered against "
                           "the previous step's graph replay; loss read back every step; "
                           "CUDA events around K consecutive steps",
                    "serial": {"value": e2e_serial, "ms_per_step": e2e_serial_ms,
                               "how": "copies, then the replay, per step on one stream"}},
            "gpu_launches": int(launches),
            "launches_per_step": int(launches) // max(1, args.steps),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clocks.summary(clocks.marks.get("t0", 0), clocks.marks.get("t1", 0)),
            "configs": configs,
            "train_iteration": train_iter,
            "loss": loss_res,
            "densify": densify,
            "scene_file": scene_file,
            "viewer": viewer,
            "kernels_ms_per_step": {k: round(v, 4) for k, v in
                                    sorted(kernel_ms.items(), key=lambda x: -x[1])},
            "isects": n_isects, "visible": n_visible, "pairs": pairs,
            "evaluated_pairs": eval_pairs, "backward_pairs": bwd_pairs,
            "wall_s_timed": wall,
            "eager": {"value": 1000.0 / eager_ms, "unit": "it/s", "ms_per_step": eager_ms,
                      "what": "the same fused step launched kernel by kernel (no graph)"},
            "dropin": {"value": 1000.0 / d_ms, "unit": "it/s", "ms_per_step": d_ms,
                       "render_fps": 1000.0 / d_fwd_ms, "kernels_ms_per_step": d_kernels,
                       "what": "the same step through the drop-in gsplat operators"},
            "ref_gpu": ref_gpu,
            # the headline figures last, where a reader of the line's tail finds them
            "summary": headline_summary(value, e2e_val, 1000.0 / fwd_ms, d_ms, d_fwd_ms,
                                        ref_gpu, roofline, configs),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
