"""numpy front end of the CPU oracle (test infrastructure only).

Every function mirrors one reference operator on the rasteriser path and runs
the C++ restatement in oracle/ubs_oracle.cpp.  dtype float32 mirrors the
reference's FP32 kernels; float64 is used for finite-difference checks.
Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use this.
"""
import ctypes
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import build_oracle  # noqa: E402

_lib = None
_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_U32 = ctypes.c_uint32


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build_oracle.build())
        for s, ft in (("f32", ctypes.c_float), ("f64", ctypes.c_double)):
            g = lambda n: getattr(_lib, "ubso_%s_%s" % (n, s))  # noqa: E731
            g("rotmat_fwd").argtypes = [_I64, _P, _I64, _P]
            g("rotmat_bwd").argtypes = [_I64, _P, _P]
            g("covar_fwd").argtypes = [_I64, _I, _P, _P, _P, _P, _P, _I, _I, _P]
            g("covar_bwd").argtypes = [_I64, _I, _P, _P, _P, _P, _P, _I, _I, _P, _P, _P, _P]
            g("cond_fwd").argtypes = [_I64, _I, _P, _P, _P, _P, _P, _P, _P, _P]
            g("cond_bwd").argtypes = [_I64, _I] + [_P] * 12 + [_I]
            g("project_fwd").argtypes = ([_I, _I64] + [_P] * 6 + [_I, _I, ft, ft, ft, ft]
                                         + [_P] * 5)
            g("project_bwd").argtypes = ([_I, _I64] + [_P] * 6 + [_I, _I, ft] + [_P] * 12)
            g("raster_fwd").argtypes = ([_I, _I64, _I, _I64] + [_P] * 7
                                        + [_I, _I, _I, _I, _I] + [_P] * 5 + [_I])
            g("raster_bwd").argtypes = ([_I, _I64, _I, _I64] + [_P] * 7
                                        + [_I, _I, _I, _I, _I] + [_P] * 11 + [_I])
        _lib.ubso_isect_count.argtypes = [_I, _I64, _P, _P, _U32, _U32, _U32, _P]
        _lib.ubso_isect_count.restype = _I64
        _lib.ubso_isect_emit_sort.argtypes = [_I, _I64, _P, _P, _P, _U32, _U32, _U32, _P,
                                              _I64, _I, _P, _P]
        _lib.ubso_offset_encode.argtypes = [_I64, _P, _I, _U32, _U32, _P]
        _lib.ubso_num_threads.restype = _I
        _lib.ubso_set_threads.argtypes = [_I]
    return _lib


def num_threads():
    return lib().ubso_num_threads()


def set_threads(n):
    lib().ubso_set_threads(int(n))


def _sfx(dtype):
    return "f64" if np.dtype(dtype) == np.float64 else "f32"


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _fn(name, dtype):
    return getattr(lib(), "ubso_%s_%s" % (name, _sfx(dtype)))


def l_triangle_to_rotmat(l, dtype=np.float32):
    l = _c(l, dtype)
    n = l.shape[0]
    R = np.zeros((n, 3, 3), dtype)
    _fn("rotmat_fwd", dtype)(n, _p(l), l.shape[1], _p(R))
    return R


def l_triangle_to_rotmat_bwd(v_R, dtype=np.float32):
    v_R = _c(v_R, dtype)
    n = v_R.shape[0]
    out = np.zeros((n, 3), dtype)
    _fn("rotmat_bwd", dtype)(n, _p(v_R), _p(out))
    return out


def rot_scale_l_triangle_to_covar(rot, scale, l_tri, rest_i, rest_j, spatial_block=False,
                                  dtype=np.float32):
    rot, scale, l_tri = _c(rot, dtype), _c(scale, dtype), _c(l_tri, dtype)
    ri, rj = _c(rest_i, np.int32), _c(rest_j, np.int32)
    n, D = scale.shape
    dim = 3 if (spatial_block or D == 3) else D
    out = np.zeros((n, dim, dim), dtype)
    _fn("covar_fwd", dtype)(n, D, _p(rot), _p(scale), _p(l_tri), _p(ri), _p(rj), len(ri),
                            int(spatial_block), _p(out))
    return out


def rot_scale_l_triangle_to_covar_bwd(rot, scale, l_tri, rest_i, rest_j, v_covar,
                                      spatial_block=False, dtype=np.float32):
    rot, scale, l_tri = _c(rot, dtype), _c(scale, dtype), _c(l_tri, dtype)
    ri, rj = _c(rest_i, np.int32), _c(rest_j, np.int32)
    v_covar = _c(v_covar, dtype)
    n, D = scale.shape
    vr = np.zeros((n, 3, 3), dtype)
    vs = np.zeros((n, D), dtype)
    vl = np.zeros((n, D * (D - 1) // 2), dtype)
    _fn("covar_bwd", dtype)(n, D, _p(rot), _p(scale), _p(l_tri), _p(ri), _p(rj), len(ri),
                            int(spatial_block), _p(v_covar), _p(vr), _p(vs), _p(vl))
    return vr, vs, vl


def cond_mean_convariance_opacity(means, covars, opacities, betas, query, dtype=np.float32):
    means, covars = _c(means, dtype), _c(covars, dtype)
    opacities, betas, query = _c(opacities, dtype), _c(betas, dtype), _c(query, dtype)
    n, D = means.shape
    om = np.zeros((n, 3), dtype)
    oV = np.zeros((n, 3, 3), dtype)
    oo = np.zeros((n, 1), dtype)
    _fn("cond_fwd", dtype)(n, D, _p(means), _p(covars), _p(opacities), _p(betas), _p(query),
                           _p(om), _p(oV), _p(oo))
    return om, oV, oo


def cond_mean_convariance_opacity_bwd(means, covars, opacities, betas, query, v_m, v_V, v_o,
                                      dtype=np.float32, exact=False):
    """exact=False reproduces the reference CUDA backward (including its
    Cholesky-backward transposition); exact=True gives the true gradient."""
    args = [_c(a, dtype) for a in (means, covars, opacities, betas, query, v_m, v_V, v_o)]
    n, D = args[0].shape
    gm = np.zeros((n, D), dtype)
    gV = np.zeros((n, D, D), dtype)
    go = np.zeros((n, 1), dtype)
    gb = np.zeros((n, D - 3), dtype)
    _fn("cond_bwd", dtype)(n, D, *[_p(a) for a in args], _p(gm), _p(gV), _p(go), _p(gb),
                           int(exact))
    return gm, gV, go, gb


def fully_fused_projection(means, covars6, quats, scales, viewmats, Ks, width, height,
                           eps2d=0.3, near_plane=0.01, far_plane=1e10, radius_clip=0.0,
                           calc_compensations=False, dtype=np.float32):
    means = _c(means, dtype)
    covars6 = None if covars6 is None else _c(covars6, dtype)
    quats = None if quats is None else _c(quats, dtype)
    scales = None if scales is None else _c(scales, dtype)
    viewmats, Ks = _c(viewmats, dtype), _c(Ks, dtype)
    N, C = means.shape[0], viewmats.shape[0]
    radii = np.zeros((C, N), np.int32)
    m2 = np.zeros((C, N, 2), dtype)
    d = np.zeros((C, N), dtype)
    cn = np.zeros((C, N, 3), dtype)
    cp = np.zeros((C, N), dtype) if calc_compensations else None
    _fn("project_fwd", dtype)(C, N, _p(means), _p(covars6), _p(quats), _p(scales), _p(viewmats),
                              _p(Ks), int(width), int(height), eps2d, near_plane, far_plane,
                              radius_clip, _p(radii), _p(m2), _p(d), _p(cn), _p(cp))
    return radii, m2, d, cn, cp


def fully_fused_projection_bwd(means, covars6, quats, scales, viewmats, Ks, width, height,
                               eps2d, radii, conics, comps, v_means2d, v_depths, v_conics,
                               v_comps=None, dtype=np.float32):
    means = _c(means, dtype)
    covars6 = None if covars6 is None else _c(covars6, dtype)
    quats = None if quats is None else _c(quats, dtype)
    scales = None if scales is None else _c(scales, dtype)
    viewmats, Ks = _c(viewmats, dtype), _c(Ks, dtype)
    radii = _c(radii, np.int32)
    conics = _c(conics, dtype)
    comps = None if comps is None else _c(comps, dtype)
    v_means2d, v_conics = _c(v_means2d, dtype), _c(v_conics, dtype)
    v_depths = None if v_depths is None else _c(v_depths, dtype)
    v_comps = None if v_comps is None else _c(v_comps, dtype)
    N, C = means.shape[0], viewmats.shape[0]
    vm = np.zeros((N, 3), dtype)
    vc6 = np.zeros((N, 6), dtype) if covars6 is not None else None
    vq = np.zeros((N, 4), dtype) if covars6 is None else None
    vs = np.zeros((N, 3), dtype) if covars6 is None else None
    vv = np.zeros((C, 4, 4), dtype)
    _fn("project_bwd", dtype)(C, N, _p(means), _p(covars6), _p(quats), _p(scales), _p(viewmats),
                              _p(Ks), int(width), int(height), eps2d, _p(radii), _p(conics),
                              _p(comps), _p(v_means2d), _p(v_depths), _p(v_conics), _p(v_comps),
                              _p(vm), _p(vc6), _p(vq), _p(vs), _p(vv))
    return vm, vc6, vq, vs, vv


def isect_tiles(means2d, radii, depths, tile_size, tile_width, tile_height, sort=True):
    means2d = _c(means2d, np.float32)
    radii = _c(radii, np.int32)
    depths = _c(depths, np.float32)
    C, N = radii.shape
    tpg = np.zeros((C, N), np.int32)
    L = lib()
    n = L.ubso_isect_count(C, N, _p(means2d), _p(radii), tile_size, tile_width, tile_height,
                           _p(tpg))
    ids = np.zeros(n, np.int64)
    fl = np.zeros(n, np.int32)
    L.ubso_isect_emit_sort(C, N, _p(means2d), _p(radii), _p(depths), tile_size, tile_width,
                           tile_height, _p(tpg), n, int(sort), _p(ids), _p(fl))
    return tpg, ids, fl


def isect_offset_encode(isect_ids, n_cameras, tile_width, tile_height):
    isect_ids = _c(isect_ids, np.int64)
    out = np.zeros((n_cameras, tile_height, tile_width), np.int32)
    lib().ubso_offset_encode(len(isect_ids), _p(isect_ids), n_cameras, tile_width, tile_height,
                             _p(out))
    return out


def rasterize_to_pixels(means2d, conics, colors, opacities, betas, width, height, tile_size,
                        isect_offsets, flatten_ids, backgrounds=None, masks=None,
                        dtype=np.float32, row_step=1, row_offset=0, out=None):
    """row_step > 1 blends only the tile rows ty with ty % row_step ==
    row_offset (a timing sample); `out` = (colors, alphas, last_ids) to write
    into instead of new zeroed arrays (rows not blended are left as they are)."""
    means2d, conics, colors = _c(means2d, dtype), _c(conics, dtype), _c(colors, dtype)
    opacities, betas = _c(opacities, dtype), _c(betas, dtype)
    offs = _c(isect_offsets, np.int32)
    fl = _c(flatten_ids, np.int32)
    bg = None if backgrounds is None else _c(backgrounds, dtype)
    mk = None if masks is None else _c(masks, np.uint8)
    C, th, tw = offs.shape
    N, cd = colors.shape[1], colors.shape[2]
    if out is None:
        oc = np.zeros((C, height, width, cd), dtype)
        oa = np.zeros((C, height, width, 1), dtype)
        li = np.zeros((C, height, width), np.int32)
    else:
        oc, oa, li = out
    _fn("raster_fwd", dtype)(C, N, cd, len(fl), _p(means2d), _p(conics), _p(colors),
                             _p(opacities), _p(betas), _p(bg), _p(mk), int(width), int(height),
                             int(tile_size), tw, th, _p(offs), _p(fl), _p(oc), _p(oa), _p(li),
                             int(row_step) | (int(row_offset) << 16))
    return oc, oa, li


def rasterize_to_pixels_bwd(means2d, conics, colors, opacities, betas, width, height,
                            tile_size, isect_offsets, flatten_ids, render_alphas, last_ids,
                            v_colors, v_alphas, backgrounds=None, masks=None, dtype=np.float32,
                            row_step=1, row_offset=0, out=None):
    """`out` = (v_means2d, v_conics, v_colors, v_opacities, v_betas) to add
    into instead of new zeroed arrays."""
    means2d, conics, colors = _c(means2d, dtype), _c(conics, dtype), _c(colors, dtype)
    opacities, betas = _c(opacities, dtype), _c(betas, dtype)
    offs = _c(isect_offsets, np.int32)
    fl = _c(flatten_ids, np.int32)
    bg = None if backgrounds is None else _c(backgrounds, dtype)
    mk = None if masks is None else _c(masks, np.uint8)
    ra, li = _c(render_alphas, dtype), _c(last_ids, np.int32)
    vc, va = _c(v_colors, dtype), _c(v_alphas, dtype)
    C, th, tw = offs.shape
    N, cd = colors.shape[1], colors.shape[2]
    if out is None:
        vm2 = np.zeros((C, N, 2), dtype)
        vcn = np.zeros((C, N, 3), dtype)
        vcol = np.zeros((C, N, cd), dtype)
        vo = np.zeros((C, N), dtype)
        vb = np.zeros((C, N), dtype)
    else:
        vm2, vcn, vcol, vo, vb = out
    _fn("raster_bwd", dtype)(C, N, cd, len(fl), _p(means2d), _p(conics), _p(colors),
                             _p(opacities), _p(betas), _p(bg), _p(mk), int(width), int(height),
                             int(tile_size), tw, th, _p(offs), _p(fl), _p(ra), _p(li), _p(vc),
                             _p(va), _p(vm2), _p(vcn), _p(vcol), _p(vo), _p(vb),
                             int(row_step) | (int(row_offset) << 16))
    return vm2, vcn, vcol, vo, vb


# ------------------------------------------------------------------- loss ---
SSIM_RADIUS = 5
SSIM_C1 = 0.01 ** 2
SSIM_C2 = 0.03 ** 2


def ssim_window():
    """Normalised 11-tap Gaussian of sigma 1.5, FP64 (utils/loss_utils.py:26-42
    builds the same window, rounded to float32, as an outer product)."""
    d = np.arange(2 * SSIM_RADIUS + 1, dtype=np.float64) - SSIM_RADIUS
    g = np.exp(-d * d / (2 * 1.5 ** 2))
    return g / g.sum()


def _corr(a, g, axis):
    """Zero-padded 'same' correlation of `a` with the symmetric window `g`
    along `axis` (F.conv2d with padding 5, utils/loss_utils.py:57-73)."""
    a = np.moveaxis(a, axis, -1)
    n = a.shape[-1]
    pad = np.pad(a, [(0, 0)] * (a.ndim - 1) + [(SSIM_RADIUS, SSIM_RADIUS)])
    out = np.zeros_like(a)
    for t in range(len(g)):
        out += g[t] * pad[..., t:t + n]
    return np.moveaxis(out, -1, axis)


def _blur(a, g):
    return _corr(_corr(a, g, -1), g, -2)


def ssim_loss(img, gt, padding="same", w_l1=0.0, w_ssim=1.0, w_const=0.0):
    """FP64 restatement of the training loss  w_l1 mean|img - gt| +
    w_ssim mean(SSIM map) + w_const  and its gradient w.r.t. img.

    img, gt: [N, C, H, W].  The map is utils/loss_utils.py:56-80's: windowed
    means, variances and covariance with zero padding, C1 = 0.01^2,
    C2 = 0.03^2; "valid" averages it over the points >= 5 pixels from every
    edge (the fused_ssim package's padding="valid"); train.py:117-121 forms the
    reference's loss as (w_l1, w_ssim, w_const) = (1 - l, -l, l).
    The gradient is the analytic chain rule through the five windowed moments
    (checked against finite differences and the reference's autograd in the
    tests).  Returns (mean map, mean |img - gt|, loss, d loss / d img)."""
    x = np.asarray(img, np.float64)
    y = np.asarray(gt, np.float64)
    g = ssim_window()
    mx, my = _blur(x, g), _blur(y, g)
    exx, eyy, exy = _blur(x * x, g), _blur(y * y, g), _blur(x * y, g)
    vx, vy, cxy = exx - mx * mx, eyy - my * my, exy - mx * my
    A1, A2 = 2 * mx * my + SSIM_C1, 2 * cxy + SSIM_C2
    B1, B2 = mx * mx + my * my + SSIM_C1, vx + vy + SSIM_C2
    smap = A1 * A2 / (B1 * B2)
    H, W = x.shape[-2:]
    mask = np.ones(x.shape, bool)
    if padding == "valid":
        r = SSIM_RADIUS
        mask[...] = False
        mask[..., r:H - r, r:W - r] = True
    elif padding != "same":
        raise ValueError(padding)
    ms = smap[mask].mean()
    ml = np.abs(x - y).mean()
    loss = w_l1 * ml + w_ssim * ms + w_const
    # d map / d (mx, E[x^2], E[xy]) with the E[.] moments free
    d0 = 2 * my * (A2 - A1) / (B1 * B2) - 2 * mx * smap * (1 / B1 - 1 / B2)
    d1 = -smap / B2
    d2 = 2 * A1 / (B1 * B2)
    scale = w_ssim / mask.sum() * mask
    grad = _blur(d0 * scale, g) + 2 * x * _blur(d1 * scale, g) + y * _blur(d2 * scale, g)
    grad += w_l1 / x.size * np.sign(x - y)
    return ms, ml, loss, grad


# ------------------------------------------------------ MCMC densification ---
MCMC_NAMES = ("xyz", "mean", "rgb", "opacity", "beta", "scale", "l_triangle")
_F32_EPS = np.float32(np.finfo(np.float32).eps)


def mcmc_split_opacity(raw_opacity, count):
    """Raw opacity of a primitive sampled `count` times, shared by it and its
    copies (scene/beta_model.py:553-562, FP32):
    logit(clamp(1 - (1 - sigmoid(raw))^(1 / (count + 1)), 0.005, 1 - eps))."""
    raw = np.asarray(raw_opacity, np.float32)
    o = (np.float32(1) / (np.float32(1) + np.exp(-raw))).astype(np.float32)
    e = (np.float32(1) / (np.asarray(count) + 1).astype(np.float32)).astype(np.float32)
    new = (np.float32(1) - np.power(np.float32(1) - o, e)).astype(np.float32)
    new = np.minimum(np.maximum(new, np.float32(0.005)), np.float32(1) - _F32_EPS)
    return np.log(new / (np.float32(1) - new)).astype(np.float32)


def mcmc_relocate(params, moments, dead, src):
    """BetaModel.relocate_gs (scene/beta_model.py:585-621) given the sampled
    live indices `src` (one per dead primitive, in index order): every dead
    primitive becomes a copy of its source with the split opacity, the sources
    take that opacity too, and the sources' Adam moments are zeroed (the dead
    slots keep theirs, as in the reference).  params: name -> [N, c];
    moments: name -> (exp_avg, exp_avg_sq).  Returns new dicts."""
    dead_idx = np.nonzero(np.asarray(dead))[0]
    src = np.asarray(src, np.int64)
    out = {k: np.array(v, np.float32, copy=True) for k, v in params.items()}
    mom = {k: (np.array(m, np.float32, copy=True), np.array(v, np.float32, copy=True))
           for k, (m, v) in moments.items()}
    if len(dead_idx) == 0 or len(src) == 0:
        return out, mom
    N = out["opacity"].shape[0]
    count = np.bincount(src, minlength=N)
    new_op = mcmc_split_opacity(out["opacity"][src, 0], count[src])
    for k in params:
        out[k][dead_idx] = params[k][src]
    out["opacity"][dead_idx, 0] = new_op
    out["opacity"][src] = out["opacity"][dead_idx]
    for k, (m, v) in mom.items():
        m[src] = 0
        v[src] = 0
    return out, mom


def mcmc_add(params, moments, src):
    """BetaModel.add_new_gs (scene/beta_model.py:623-658) given the sampled
    indices `src` (one per new primitive): the new primitives, appended in
    order, copy their sources with the split opacity; the sources take that
    opacity; the grown Adam moments are zero for the new rows and at the
    sources."""
    src = np.asarray(src, np.int64)
    N = params["opacity"].shape[0]
    count = np.bincount(src, minlength=N)
    new_op = mcmc_split_opacity(params["opacity"][src, 0], count[src])
    new = {k: np.array(v, np.float32)[src] for k, v in params.items()}
    new["opacity"][:, 0] = new_op
    out = {k: np.array(v, np.float32, copy=True) for k, v in params.items()}
    out["opacity"][src, 0] = new_op
    out = {k: np.concatenate([out[k], new[k]], 0) for k in params}
    mom = {}
    for k, (m, v) in moments.items():
        m2 = np.concatenate([m, np.zeros_like(new[k])], 0).astype(np.float32)
        v2 = np.concatenate([v, np.zeros_like(new[k])], 0).astype(np.float32)
        m2[src] = 0
        v2[src] = 0
        mom[k] = (m2, v2)
    return out, mom


def mcmc_add_count(n_prims, cap_max):
    """Primitives add_new_gs appends (scene/beta_model.py:624-626)."""
    return max(0, min(int(cap_max), int(1.02 * n_prims)) - int(n_prims))


def xyz_covariance(raw_scale, l_triangle):
    """Spatial 3 x 3 block of the primitive covariance (get_xyz_covariance,
    scene/beta_model.py:144-152): R diag(s^2) R^T with s = softplus of the
    first three raw scales and R = I + A from l_triangle[:, :3]."""
    s = np.log1p(np.exp(np.asarray(raw_scale, np.float64)[:, :3]))
    R = l_triangle_to_rotmat(np.asarray(l_triangle, np.float64)[:, :3], dtype=np.float64)
    M = R * s[:, None, :]
    return M @ np.transpose(M, (0, 2, 1))


def mcmc_perturb_xyz(xyz, raw_opacity, raw_scale, l_triangle, noise, factor):
    """train.py:164-171: xyz + Sigma_xyz (noise (1 - sigmoid(raw_opacity))^100
    factor), factor = noise_lr * xyz_lr, for given standard-normal noise."""
    o = 1.0 / (1.0 + np.exp(-np.asarray(raw_opacity, np.float64)))
    n = np.asarray(noise, np.float64) * (1.0 - o) ** 100 * factor
    cov = xyz_covariance(raw_scale, l_triangle)
    return np.asarray(xyz, np.float64) + np.einsum("nij,nj->ni", cov, n)


# ------------------------------------------------------------ scene files ---
def ply_attribute_names(n_beta, n_mean, n_scale, n_ltri):
    """construct_list_of_attributes (scene/beta_model.py:286-296)."""
    return (["x", "y", "z", "red", "green", "blue", "opacity"]
            + ["beta_%d" % i for i in range(n_beta)] + ["mean_%d" % i for i in range(n_mean)]
            + ["scale_%d" % i for i in range(n_scale)]
            + ["l_triangle_%d" % i for i in range(n_ltri)])


def ply_bytes(params, names=None, comments=()):
    """The bytes of the reference's scene file (save_ply, beta_model.py:298-320:
    one vertex element, float32 properties, binary little-endian, written by
    plyfile) for raw parameters {xyz, mean, rgb, opacity, beta, scale,
    l_triangle}; `names` reorders or extends the properties (a name not in the
    default list is written as zeros) and `comments` adds comment lines."""
    cols = {}
    p = {}
    for k, v in params.items():
        a = np.asarray(v, np.float32)
        p[k] = a[:, None] if a.ndim == 1 else a.reshape(a.shape[0], -1 if a.shape[0] else
                                                        int(np.prod(a.shape[1:])))
    for i, c in enumerate("xyz"):
        cols[c] = p["xyz"][:, i]
    for i, c in enumerate(("red", "green", "blue")):
        cols[c] = p["rgb"][:, i]
    cols["opacity"] = p["opacity"][:, 0]
    for fam, key in (("beta", "beta"), ("mean", "mean"), ("scale", "scale"),
                     ("l_triangle", "l_triangle")):
        for i in range(p[key].shape[1]):
            cols["%s_%d" % (fam, i)] = p[key][:, i]
    default = ply_attribute_names(p["beta"].shape[1], p["mean"].shape[1], p["scale"].shape[1],
                                  p["l_triangle"].shape[1])
    names = list(default if names is None else names)
    n = p["xyz"].shape[0]
    head = "ply\nformat binary_little_endian 1.0\n"
    head += "".join("comment %s\n" % c for c in comments)
    head += "element vertex %d\n" % n
    head += "".join("property float %s\n" % nm for nm in names) + "end_header\n"
    rec = np.zeros((n, len(names)), "<f4")
    for j, nm in enumerate(names):
        if nm in cols:
            rec[:, j] = cols[nm]
    return head.encode() + rec.tobytes()


def ply_parse(data):
    """Raw parameters read from scene-file bytes the way load_ply
    (beta_model.py:322-404) reads them: by property name, each of the beta_,
    mean_, scale_, l_triangle families sorted by numeric suffix."""
    end = data.index(b"end_header\n") + len(b"end_header\n")
    lines = data[:end].decode().splitlines()
    assert lines[0] == "ply" and lines[1] == "format binary_little_endian 1.0"
    n = None
    names = []
    for ln in lines[2:]:
        w = ln.split()
        if w[0] == "element" and w[1] == "vertex":
            n = int(w[2])
        elif w[0] == "property":
            assert w[1] in ("float", "float32")
            names.append(w[2])
    rec = np.frombuffer(data[end:end + n * len(names) * 4], "<f4").reshape(n, len(names))
    col = {nm: rec[:, i] for i, nm in enumerate(names)}

    def fam(prefix):
        sel = sorted([nm for nm in names if nm.startswith(prefix)],
                     key=lambda s: int(s.split("_")[-1]))
        return np.stack([col[s] for s in sel], 1) if sel else np.zeros((n, 0), np.float32)

    return {"xyz": np.stack([col["x"], col["y"], col["z"]], 1),
            "rgb": np.stack([col["red"], col["green"], col["blue"]], 1),
            "opacity": col["opacity"][:, None].copy(),
            "mean": fam("mean_"), "beta": fam("beta_"), "scale": fam("scale_"),
            "l_triangle": fam("l_triangle")}
