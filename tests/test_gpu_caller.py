"""The reference's own caller against this repository's drop-in operators.

tests/golden/make_caller_golden.py ran the reference model's render
(scene/beta_model.py:660-722) UNCHANGED on the CPU, with its gsplat imports
bound to recorders that check every call against the signatures of this
repository's functions and keep the arguments.  Here those recorded calls --
the same functions, positional and keyword arguments as BetaModel passed them
(a 6-D model, a 7-D model with a timestamp, and a render with a primitive
mask) -- are replayed on the GPU through this repository's operators and
through the reference's CUDA kernels (oracle/ref_gpu.py) on the same inputs:

* l_triangle_to_rotmat, rot_scale_l_triangle_to_covar and
  cond_mean_convariance_opacity: bit-exact;
* rasterization: radii, isect_ids, flatten_ids and isect_offsets bit-exact,
  image and alpha within 1e-5, and the gradients of a weighted image sum with
  respect to every differentiable argument (means, covars, opacities, betas,
  colors) within 1e-4 relative (L2).
"""
import inspect
import math
import os

import numpy as np
import pytest
import torch

import ref_gpu
from gsplat.cuda._wrapper import (cond_mean_convariance_opacity, l_triangle_to_rotmat,
                                  rot_scale_l_triangle_to_covar)
from gsplat.rendering import rasterization

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_gpu.available(),
                                 reason="reference kernels not built (oracle/build_ref.py)")]
DEV = "cuda"
FIX = np.load(os.path.join(os.path.dirname(__file__), "golden", "caller.npz"))
CASES = ("d6", "d7", "d6m")
OURS = {"l_triangle_to_rotmat": l_triangle_to_rotmat,
        "rot_scale_l_triangle_to_covar": rot_scale_l_triangle_to_covar,
        "cond_mean_convariance_opacity": cond_mean_convariance_opacity,
        "rasterization": rasterization}


@pytest.fixture(scope="module")
def k():
    return ref_gpu.RefKernels()


def recorded(tag):
    """[(function name, keyword names, {argument: value})] in call order."""
    out = []
    for i, name in enumerate(FIX[tag + "/calls"]):
        pre = "%s/%d/" % (tag, i)
        args = {}
        for key in FIX.files:
            if key.startswith(pre) and key != pre + "keywords":
                v = FIX[key]
                if v.dtype.kind in "fi" and v.ndim > 0:
                    # row-major copies: a transposed argument (the model passes
                    # world_view_transform.transpose(0, 1)) is stored column-major
                    v = torch.from_numpy(np.ascontiguousarray(v)).to(DEV)
                else:
                    v = v.item()
                args[key[len(pre):]] = v
        out.append((str(name), [str(s) for s in FIX[pre + "keywords"]], args))
    return out


def invoke(name, kwnames, args, override=None):
    """Call our function as the model did: arguments it passed by keyword by
    keyword, the others positionally in parameter order."""
    fn = OURS[name]
    a = dict(args, **(override or {}))
    pos = [a[p] for p in inspect.signature(fn).parameters if p in a and p not in kwnames]
    return fn(*pos, **{n: a[n] for n in kwnames})


def rel_l2(a, b):
    a, b = a.detach().double(), b.detach().double()
    return float((a - b).norm() / b.norm().clamp_min(1e-30))


@pytest.mark.parametrize("tag", CASES)
def test_model_call_sequence(tag):
    assert [c[0] for c in recorded(tag)] == ["l_triangle_to_rotmat",
                                             "rot_scale_l_triangle_to_covar",
                                             "cond_mean_convariance_opacity", "rasterization"]


@pytest.mark.parametrize("tag", CASES)
def test_per_primitive_operators_bit_exact(k, tag):
    calls = {c[0]: c for c in recorded(tag)}
    with torch.no_grad():
        name, kw, a = calls["l_triangle_to_rotmat"]
        assert torch.equal(invoke(name, kw, a), k.rotmat_fwd(a["l_triangle"].contiguous()))
        name, kw, a = calls["rot_scale_l_triangle_to_covar"]
        ours = invoke(name, kw, a)
        ref = k.covar_fwd(a["rot"].contiguous(), a["scale"].contiguous(),
                          a["l_triangle"].contiguous(), a["rest_i"], a["rest_j"])
        assert torch.equal(ours, ref), int((ours != ref).sum())
        name, kw, a = calls["cond_mean_convariance_opacity"]
        ours = invoke(name, kw, a)
        ref = k.cond_fwd(*[a[n].contiguous() for n in
                           ("means", "covars", "opacities", "betas", "query")])
        for o, r in zip(ours, ref):
            assert torch.equal(o, r)


def reference_rasterization(rp, a, leaves):
    """The reference's rasterization() steps for this call on its own kernels:
    upper-triangle gather, projection, intersections + stable sort, offsets,
    blend (rendering.py:42-232, RGB mode, one camera)."""
    W, H = int(a["width"]), int(a["height"])
    means, covars, opac, betas, colors = leaves
    c6 = covars[..., [0, 0, 0, 1, 1, 2], [0, 1, 2, 1, 2, 2]]
    radii, m2, d, cn = rp.Proj.apply(means, c6, a["viewmats"], a["Ks"], W, H)
    tw, th = math.ceil(W / 16), math.ceil(H / 16)
    with torch.no_grad():
        _, ids, fl = rp.k.isect_tiles(m2.detach(), radii, d.detach(), 16, tw, th)
        offs = rp.k.offset_encode(ids, 1, tw, th)
    img, alpha = rp.Raster.apply(m2, cn, colors.expand(1, -1, -1), opac.repeat(1, 1),
                                 betas.repeat(1, 1), a["backgrounds"], W, H, 16, offs, fl)
    return img, alpha, dict(radii=radii, isect_ids=ids, flatten_ids=fl, isect_offsets=offs)


@pytest.mark.parametrize("tag", CASES)
def test_rasterization_matches_reference_kernels(k, tag):
    rp = ref_gpu.RefPipeline(k)
    name, kw, a = [c for c in recorded(tag) if c[0] == "rasterization"][0]
    diff = ("means", "covars", "opacities", "betas", "colors")
    ours_in = {n: a[n].clone().requires_grad_(True) for n in diff}
    img, alpha, meta = invoke(name, kw, a, ours_in)
    ref_in = [a[n].clone().requires_grad_(True) for n in diff]
    img_r, alpha_r, meta_r = reference_rasterization(rp, a, ref_in)
    for key in ("radii", "isect_ids", "flatten_ids", "isect_offsets"):
        assert torch.equal(meta[key], meta_r[key]), key
    assert float((img - img_r).abs().max()) <= 1e-5
    assert float((alpha - alpha_r).abs().max()) <= 1e-5
    g = torch.Generator().manual_seed(7)
    wc = torch.randn(img.shape, generator=g).to(DEV)
    wa = torch.randn(alpha.shape, generator=g).to(DEV)
    ((img * wc).sum() + (alpha * wa).sum()).backward()
    ((img_r * wc).sum() + (alpha_r * wa).sum()).backward()
    for n, r in zip(diff, ref_in):
        assert rel_l2(ours_in[n].grad, r.grad) < 1e-4, n
