"""Record how the reference's own model calls the rasteriser: the calls
BetaModel.render (scene/beta_model.py:660-722) makes into gsplat, with the
arguments it passes, for a 6-D and a 7-D model.

The reference model is loaded from a checkout of the reference on the CPU (its
absent imports stubbed, as make_mcmc_golden.py does) and run UNCHANGED.  The
four gsplat names it imports -- l_triangle_to_rotmat,
rot_scale_l_triangle_to_covar, cond_mean_convariance_opacity (gsplat.cuda.
_wrapper) and rasterization (gsplat.rendering) -- are bound to recorders that

  1. bind the call against the signature of THIS repository's function of the
     same name (inspect.signature(...).bind raises if BetaModel passes an
     argument our drop-in does not accept), and record the bound arguments;
  2. return the reference's own CPU results for the per-primitive operators
     (submodules/gsplat/cuda/_torch_impl.py) so the model proceeds on genuine
     values, and, for rasterization (which has no CPU implementation in the
     reference), outputs of the right shapes.

The recorded calls (function, argument names, values) go to caller.npz next
to this script.  tests/test_gpu_caller.py replays them through this
repository's operators and through the reference's CUDA kernels on the GPU.

Usage:  python tests/golden/make_caller_golden.py /path/to/reference
"""
import inspect
import math
import os
import sys
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("UBS_REFERENCE_ROOT")
if not REF:
    sys.exit("usage: %s /path/to/reference (or set UBS_REFERENCE_ROOT)" % sys.argv[0])
sys.path.insert(0, HERE)
import make_mcmc_golden as mm  # noqa: E402  (its stubbed loader of BetaModel)

W, H = 96, 64
NAMES = ("xyz", "mean", "scale", "l_triangle", "opacity", "beta", "rgb")


def our_signatures():
    """Signatures of this repository's drop-in functions (imported without a
    GPU: nothing is called)."""
    pkg = os.path.join(ROOT, "universal-beta-splatting_gb300")
    saved = {k: v for k, v in sys.modules.items() if k == "gsplat" or k.startswith("gsplat.")}
    for k in saved:
        del sys.modules[k]
    sys.path.insert(0, pkg)
    try:
        from gsplat.cuda import _wrapper as w
        from gsplat import rendering as r
        sigs = {n: inspect.signature(getattr(w, n)) for n in
                ("l_triangle_to_rotmat", "rot_scale_l_triangle_to_covar",
                 "cond_mean_convariance_opacity")}
        sigs["rasterization"] = inspect.signature(r.rasterization)
    finally:
        sys.path.remove(pkg)
        for k in [k for k in sys.modules if k == "gsplat" or k.startswith("gsplat.")]:
            del sys.modules[k]
        sys.modules.update(saved)
    return sigs


def make_model(BetaModel, D, N, seed):
    g = torch.Generator().manual_seed(seed)
    m = object.__new__(BetaModel)
    m.input_dim = D
    m.setup_functions()
    K = D - 3
    xyz = (torch.rand(N, 3, generator=g) * 2 - 1)
    mean = torch.rand(N, K, generator=g) * 2 - 1
    if D == 7:
        mean[:, 3] = torch.rand(N, generator=g)
    # spatial scales of a few pixels at this resolution; angular scales ~1
    s = torch.cat([torch.exp(torch.randn(N, 3, generator=g) * 0.4 - 3.0),
                   1.0 + 0.05 * torch.randn(N, K, generator=g)], 1)
    raw = {"xyz": xyz, "mean": mean, "scale": s + torch.log(-torch.expm1(-s)),
           "l_triangle": torch.randn(N, D * (D - 1) // 2, generator=g) * 0.1,
           "opacity": torch.randn(N, 1, generator=g),
           "beta": torch.cat([torch.randn(N, 1, generator=g) * 0.3,
                              torch.randn(N, K, generator=g) * 0.5], 1),
           "rgb": torch.rand(N, 3, generator=g)}
    for k, v in raw.items():
        setattr(m, "_" + k, torch.nn.Parameter(v.contiguous()))
    ti, tj = torch.tril_indices(D, D, offset=-1)
    rest = (ti >= 3) | (tj >= 3)
    m.rest_i, m.rest_j = ti[rest].to(torch.int32), tj[rest].to(torch.int32)
    m.background = torch.tensor([0.1, 0.2, 0.3])
    return m, raw


def make_camera(seed, timestamp):
    """The attributes BetaModel.render reads from the reference's Camera
    (scene/cameras.py): FoV, size, world_view_transform (world-to-camera,
    transposed), camera_center, projection_matrix (for its device), timestamp."""
    g = torch.Generator().manual_seed(seed)
    v = torch.randn(3, generator=g, dtype=torch.float64)
    eye = v / v.norm() * 3.0
    f = -eye / eye.norm()
    r = torch.linalg.cross(f, torch.tensor([0.0, 1.0, 0.0], dtype=torch.float64))
    r = r / r.norm()
    u = torch.linalg.cross(r, f)
    Rw = torch.stack([r, -u, f], 0)
    w2c = torch.eye(4, dtype=torch.float64)
    w2c[:3, :3] = Rw
    w2c[:3, 3] = -Rw @ eye
    wvt = w2c.float().t().contiguous()
    fovx, fovy = 2 * math.atan(W / (2 * 70.0)), 2 * math.atan(H / (2 * 70.0))
    return types.SimpleNamespace(
        FoVx=fovx, FoVy=fovy, image_width=W, image_height=H, world_view_transform=wvt,
        camera_center=wvt.inverse()[3, :3], projection_matrix=torch.eye(4),
        timestamp=timestamp)


def main():
    BetaModel = mm.load_beta_model()
    mod = types.SimpleNamespace()  # assignments below go into the module's globals
    from gsplat.cuda import _torch_impl as ti
    sigs = our_signatures()
    log = []

    def recorder(name, compute):
        def call(*args, **kwargs):
            bound = sigs[name].bind(*args, **kwargs)  # TypeError if our drop-in cannot take it
            log.append((name, [k for k in kwargs], dict(bound.arguments)))
            return compute(*args, **kwargs)
        return call

    def raster_out(**kw):
        C = kw["viewmats"].shape[0]
        N = kw["means"].shape[0]
        return (torch.zeros(C, kw["height"], kw["width"], kw["colors"].shape[-1]),
                torch.zeros(C, kw["height"], kw["width"], 1),
                {"means2d": torch.zeros(C, N, 2), "radii": torch.zeros(C, N, dtype=torch.int32)})

    mod.l_triangle_to_rotmat = recorder("l_triangle_to_rotmat", ti._l_triangle_to_rotmat)
    mod.rot_scale_l_triangle_to_covar = recorder(
        "rot_scale_l_triangle_to_covar",
        lambda rot, scale, l_triangle, rest_i, rest_j, spatial_block=False:
        ti._rot_scale_l_triangle_to_covar(rot, scale, l_triangle, rest_i.long(), rest_j.long(),
                                          spatial_block))
    mod.cond_mean_convariance_opacity = recorder("cond_mean_convariance_opacity",
                                                 ti._cond_mean_convariance_opacity)
    mod.rasterization = recorder("rasterization", lambda *a, **kw: raster_out(
        **sigs["rasterization"].bind(*a, **kw).arguments))
    BetaModel.render.__globals__.update(vars(mod))

    out = {}
    cases = [("d6", 6, 400, 1, None), ("d7", 7, 350, 2, 0.35), ("d6m", 6, 400, 3, "mask")]
    for tag, D, N, seed, extra in cases:
        m, raw = make_model(BetaModel, D, N, seed)
        cam = make_camera(10 + seed, extra if isinstance(extra, float) else 0.0)
        log.clear()
        with torch.no_grad():
            if extra == "mask":
                mask = torch.rand(N, generator=torch.Generator().manual_seed(5)) < 0.7
                m.render(cam, mask=mask)
                out[tag + "/mask"] = mask.numpy()
            else:
                m.render(cam)
        for k, v in raw.items():
            out["%s/param/%s" % (tag, k)] = v.numpy()
        out[tag + "/calls"] = np.array([c[0] for c in log])
        for i, (name, kwnames, args) in enumerate(log):
            out["%s/%d/keywords" % (tag, i)] = np.array(kwnames, dtype=str)
            for a, v in args.items():
                key = "%s/%d/%s" % (tag, i, a)
                if isinstance(v, torch.Tensor):
                    out[key] = v.detach().numpy()
                else:
                    out[key] = np.array(v)
        print(tag, [c[0] for c in log])
    np.savez_compressed(os.path.join(HERE, "caller.npz"), **out)
    print("wrote caller.npz")


if __name__ == "__main__":
    main()
