"""Launch the reference's own CUDA kernels (cubins built by oracle/build_ref.py).

TEST INFRASTRUCTURE ONLY: used by GPU parity tests and by bench.py to time the
reference's plain one-view-per-launch path on the same GPU.  Kernels are loaded
with the CUDA driver API and launched with the argument lists and launch shapes
of the reference's host code:
  fully_fused_projection_fwd.cu:228 / _bwd.cu:312, isect_tiles.cu:156,197,352,
  rasterize_to_pixels_fwd.cu:269 / _bwd.cu:365,
  cond_mean_convariance_opacity_fwd.cu:334 / _bwd.cu:612,
  rot_scale_l_triangle_to_covar_fwd.cu:220 / _bwd.cu:274,
  l_triagnle_to_rotmat_fwd.cu:55 / _bwd.cu:47.
The reference sorts intersections with cub::DeviceRadixSort::SortPairs over
bits [0, 32 + tile_bits + cam_bits); here torch.sort(stable=True) on the same
non-negative keys defines the same order.
"""
import ctypes
import math
import os

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

_U32, _I32, _I64 = ctypes.c_uint32, ctypes.c_int32, ctypes.c_int64
_F32, _BOOL, _PTR = ctypes.c_float, ctypes.c_bool, ctypes.c_void_p

KERNELS = {
    # key: (cubin, unique substring of the mangled name)
    "proj_fwd": ("fully_fused_projection_fwd", "fully_fused_projection_fwd_kernelIfE"),
    "proj_bwd": ("fully_fused_projection_bwd", "fully_fused_projection_bwd_kernelIfE"),
    "isect": ("isect_tiles", "11isect_tilesIfE"),
    "offset_encode": ("isect_tiles", "19isect_offset_encodeE"),
    "raster_fwd3": ("rasterize_to_pixels_fwd", "rasterize_to_pixels_fwd_kernelILj3EfE"),
    "raster_bwd3": ("rasterize_to_pixels_bwd", "rasterize_to_pixels_bwd_kernelILj3EfE"),
    "cond_fwd": ("cond_mean_convariance_opacity_fwd",
                 "cond_mean_convariance_opacity_fwd_kernelILi8EfE"),
    "cond_bwd": ("cond_mean_convariance_opacity_bwd",
                 "cond_mean_convariance_opacity_bwd_kernelILi8EfE"),
    "covar_fwd": ("rot_scale_l_triangle_to_covar_fwd", "rot_scale_l_triangle_to_covar_fwd_kernelIfE"),
    "covar_bwd": ("rot_scale_l_triangle_to_covar_bwd", "rot_scale_l_triangle_to_covar_bwd_kernelIfE"),
    "rot_fwd": ("l_triagnle_to_rotmat_fwd", "l_triangle_to_rotmat_fwd_kernelIfE"),
    "rot_bwd": ("l_triagnle_to_rotmat_bwd", "l_triangle_to_rotmat_bwd_kernelIfE"),
}


def available():
    return all(os.path.exists(os.path.join(REF_DIR, c + ".cubin")) for c, _ in KERNELS.values())


class _Driver:
    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        cu = self.cu
        cu.cuModuleLoad.argtypes = [ctypes.POINTER(_PTR), ctypes.c_char_p]
        cu.cuModuleGetFunctionCount.argtypes = [ctypes.POINTER(ctypes.c_uint), _PTR]
        cu.cuModuleEnumerateFunctions.argtypes = [ctypes.POINTER(_PTR), ctypes.c_uint, _PTR]
        cu.cuFuncGetName.argtypes = [ctypes.POINTER(ctypes.c_char_p), _PTR]
        cu.cuLaunchKernel.argtypes = [_PTR] + [ctypes.c_uint] * 7 + [_PTR, ctypes.POINTER(_PTR),
                                                                     ctypes.POINTER(_PTR)]
        cu.cuGetErrorString.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]

    def check(self, rc, what):
        if rc != 0:
            s = ctypes.c_char_p()
            self.cu.cuGetErrorString(rc, ctypes.byref(s))
            raise RuntimeError("%s: CUDA driver error %d (%s)" % (what, rc, s.value))

    def functions(self, path):
        mod = _PTR()
        self.check(self.cu.cuModuleLoad(ctypes.byref(mod), path.encode()), "cuModuleLoad " + path)
        n = ctypes.c_uint()
        self.check(self.cu.cuModuleGetFunctionCount(ctypes.byref(n), mod), "function count")
        arr = (_PTR * n.value)()
        self.check(self.cu.cuModuleEnumerateFunctions(arr, n.value, mod), "enumerate")
        out = {}
        for f in arr:
            nm = ctypes.c_char_p()
            self.check(self.cu.cuFuncGetName(ctypes.byref(nm), f), "cuFuncGetName")
            out[nm.value.decode()] = f
        return out


class RefKernels:
    """The reference's kernels, callable on torch CUDA tensors."""

    def __init__(self):
        if not available():
            raise RuntimeError("reference cubins missing: run oracle/build_ref.py")
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current
        self.drv = _Driver()
        mods = {}
        self.fn = {}
        for key, (cubin, sub) in KERNELS.items():
            if cubin not in mods:
                mods[cubin] = self.drv.functions(os.path.join(REF_DIR, cubin + ".cubin"))
            hits = [f for n, f in mods[cubin].items() if sub in n]
            if len(hits) != 1:
                raise RuntimeError("kernel %s: %d matches for %s in %s" % (key, len(hits), sub,
                                                                            sorted(mods[cubin])))
            self.fn[key] = hits[0]

    def launch(self, key, grid, block, smem, args):
        """args: list of ctypes scalars in the kernel's parameter order."""
        vals = list(args)
        params = (_PTR * len(vals))(*[ctypes.cast(ctypes.pointer(v), _PTR) for v in vals])
        g = tuple(grid) + (1,) * (3 - len(grid))
        b = tuple(block) + (1,) * (3 - len(block))
        st = _PTR(torch.cuda.current_stream().cuda_stream)
        self.drv.check(self.drv.cu.cuLaunchKernel(self.fn[key], g[0], g[1], g[2], b[0], b[1], b[2],
                                                  smem, st, params, None), "launch " + key)

    @staticmethod
    def p(t):
        return _PTR(0 if t is None else t.data_ptr())

    # ---------------------------------------------------------------- ops
    def projection_fwd(self, means, covars6, viewmats, Ks, W, H, eps2d=0.3, near=0.01, far=1e10,
                       radius_clip=0.0, calc_comp=False):
        C, N = viewmats.shape[0], means.shape[0]
        dev = means.device
        radii = torch.empty(C, N, dtype=torch.int32, device=dev)
        m2 = torch.empty(C, N, 2, device=dev)
        d = torch.empty(C, N, device=dev)
        cn = torch.empty(C, N, 3, device=dev)
        comp = torch.zeros(C, N, device=dev) if calc_comp else None
        if C * N:
            P = self.p
            self.launch("proj_fwd", (math.ceil(C * N / 256),), (256,), 0, [
                _U32(C), _U32(N), P(means), P(covars6), P(None), P(None), P(viewmats), P(Ks),
                _I32(W), _I32(H), _F32(eps2d), _F32(near), _F32(far), _F32(radius_clip),
                _BOOL(False), P(radii), P(m2), P(d), P(cn), P(comp)])
        return radii, m2, d, cn, comp

    def projection_bwd(self, means, covars6, viewmats, Ks, W, H, eps2d, radii, conics, v_m2, v_d,
                       v_cn, want_viewmat_grad=False):
        C, N = viewmats.shape[0], means.shape[0]
        dev = means.device
        v_means = torch.zeros(N, 3, device=dev)
        v_cov = torch.zeros(N, 6, device=dev)
        v_view = torch.zeros(C, 4, 4, device=dev) if want_viewmat_grad else None
        if C * N:
            P = self.p
            self.launch("proj_bwd", (math.ceil(C * N / 256),), (256,), 0, [
                _U32(C), _U32(N), P(means), P(covars6), P(None), P(None), P(viewmats), P(Ks),
                _I32(W), _I32(H), _F32(eps2d), _BOOL(False), P(radii), P(conics), P(None),
                P(v_m2), P(v_d), P(v_cn), P(None), P(v_means), P(v_cov), P(None), P(None),
                P(v_view)])
        return v_means, v_cov, v_view

    def isect_tiles(self, means2d, radii, depths, tile_size, tw, th):
        C, N = radii.shape
        dev = means2d.device
        n_tiles = tw * th
        tile_bits = int(math.floor(math.log2(n_tiles))) + 1
        tpg = torch.empty(C, N, dtype=torch.int32, device=dev)
        P = self.p
        if C * N:
            self.launch("isect", (math.ceil(C * N / 256),), (256,), 0, [
                _U32(C), _U32(N), _U32(0), P(None), P(None), P(means2d), P(radii), P(depths),
                P(None), _U32(tile_size), _U32(tw), _U32(th), _U32(tile_bits), P(tpg), P(None),
                P(None)])
            cum = torch.cumsum(tpg.view(-1), 0)
            T = int(cum[-1].item())
        else:
            T = 0
        ids = torch.empty(T, dtype=torch.int64, device=dev)
        fl = torch.empty(T, dtype=torch.int32, device=dev)
        if T:
            self.launch("isect", (math.ceil(C * N / 256),), (256,), 0, [
                _U32(C), _U32(N), _U32(0), P(None), P(None), P(means2d), P(radii), P(depths),
                P(cum), _U32(tile_size), _U32(tw), _U32(th), _U32(tile_bits), P(None), P(ids),
                P(fl)])
            ids, order = torch.sort(ids, stable=True)
            fl = fl[order]
        return tpg, ids, fl

    def offset_encode(self, ids, C, tw, th):
        n_tiles = tw * th
        tile_bits = int(math.floor(math.log2(n_tiles))) + 1
        offs = torch.empty(C, th, tw, dtype=torch.int32, device=ids.device)
        T = ids.numel()
        if T:
            self.launch("offset_encode", (math.ceil(T / 256),), (256,), 0, [
                _U32(T), self.p(ids), _U32(C), _U32(n_tiles), _U32(tile_bits), self.p(offs)])
        else:
            offs.zero_()
        return offs

    def raster_fwd(self, means2d, conics, colors, opac, betas, bg, W, H, ts, offsets, flatten):
        C, N, ch = colors.shape
        assert ch == 3, "the reference kernels are loaded for 3 channels"
        th, tw = offsets.shape[1:]
        dev = means2d.device
        out_c = torch.empty(C, H, W, ch, device=dev)
        out_a = torch.empty(C, H, W, 1, device=dev)
        last = torch.empty(C, H, W, dtype=torch.int32, device=dev)
        P = self.p
        self.launch("raster_fwd3", (C, th, tw), (ts, ts), ts * ts * 32, [
            _U32(C), _U32(N), _U32(flatten.numel()), P(means2d), P(conics), P(colors), P(opac),
            P(betas), P(bg), P(None), _U32(W), _U32(H), _U32(ts), _U32(tw), _U32(th), P(offsets),
            P(flatten), P(out_c), P(out_a), P(last)])
        return out_c, out_a, last

    def raster_bwd(self, means2d, conics, colors, opac, betas, bg, W, H, ts, offsets, flatten,
                   render_alphas, last_ids, v_out_c, v_out_a):
        C, N, ch = colors.shape
        assert ch == 3
        th, tw = offsets.shape[1:]
        dev = means2d.device
        v_m2 = torch.zeros(C, N, 2, device=dev)
        v_cn = torch.zeros(C, N, 3, device=dev)
        v_col = torch.zeros(C, N, ch, device=dev)
        v_op = torch.zeros(C, N, device=dev)
        v_be = torch.zeros(C, N, device=dev)
        if flatten.numel():
            P = self.p
            self.launch("raster_bwd3", (C, th, tw), (ts, ts), ts * ts * (32 + 4 * ch), [
                _U32(C), _U32(N), _U32(flatten.numel()), P(means2d), P(conics), P(colors),
                P(opac), P(betas), P(bg), P(None), _U32(W), _U32(H), _U32(ts), _U32(tw), _U32(th),
                P(offsets), P(flatten), P(render_alphas), P(last_ids), P(v_out_c), P(v_out_a),
                P(v_m2), P(v_cn), P(v_col), P(v_op), P(v_be)])
        return v_m2, v_cn, v_col, v_op, v_be

    def cond_fwd(self, means, covars, opac, betas, query):
        N, D = means.shape
        dev = means.device
        om = torch.empty(N, 3, device=dev)
        oV = torch.empty(N, 3, 3, device=dev)
        oo = torch.empty(N, 1, device=dev)
        if N:
            P = self.p
            self.launch("cond_fwd", (math.ceil(N / 256),), (256,), 0, [
                _I64(N), _I64(D), P(means), P(covars), P(opac), P(betas), P(query), P(om), P(oV),
                P(oo)])
        return om, oV, oo

    def cond_bwd(self, means, covars, opac, betas, query, v_m, v_V, v_o):
        N, D = means.shape
        dev = means.device
        gm = torch.zeros(N, D, device=dev)
        gV = torch.zeros(N, D, D, device=dev)
        go = torch.zeros(N, 1, device=dev)
        gb = torch.zeros(N, D - 3, device=dev)
        if N:
            P = self.p
            self.launch("cond_bwd", (math.ceil(N / 256),), (256,), 0, [
                _I64(N), _I64(D), P(means), P(covars), P(opac), P(betas), P(query), P(v_m),
                P(v_V), P(v_o), P(gm), P(gV), P(go), P(gb)])
        return gm, gV, go, gb

    def covar_fwd(self, rot, scale, ltri, rest_i, rest_j, spatial=False):
        N, D = scale.shape
        dim = 3 if spatial else D
        out = torch.empty(N, dim, dim, device=rot.device)
        if N:
            P = self.p
            self.launch("covar_fwd", (math.ceil(N / 256),), (256,), 0, [
                _I64(N), _I64(D), P(rot), P(scale), P(ltri), P(rest_i), P(rest_j),
                _I64(rest_i.numel()), _BOOL(spatial), P(out)])
        return out

    def covar_bwd(self, rot, scale, ltri, rest_i, rest_j, v_covar, spatial=False):
        N, D = scale.shape
        dev = rot.device
        vr = torch.zeros(N, 3, 3, device=dev)
        vs = torch.zeros(N, D, device=dev)
        vl = torch.zeros(N, D * (D - 1) // 2, device=dev)
        if N:
            P = self.p
            self.launch("covar_bwd", (math.ceil(N / 256),), (256,), 0, [
                _I64(N), _I64(D), P(rot), P(scale), P(ltri), P(rest_i), P(rest_j),
                _I64(rest_i.numel()), _BOOL(spatial), P(v_covar), P(vr), P(vs), P(vl)])
        return vr, vs, vl

    def rotmat_fwd(self, l3):
        N = l3.shape[0]
        R = torch.empty(N, 3, 3, device=l3.device)
        if N:
            self.launch("rot_fwd", (math.ceil(N / 256),), (256,), 0, [_I64(N), self.p(l3),
                                                                      self.p(R)])
        return R

    def rotmat_bwd(self, v_R):
        N = v_R.shape[0]
        vl = torch.empty(N, 3, device=v_R.device)
        if N:
            self.launch("rot_bwd", (math.ceil(N / 256),), (256,), 0, [_I64(N), self.p(v_R),
                                                                      self.p(vl)])
        return vl


# ------------------------------------------------------------------------
# The reference's plain render path on its own kernels: autograd Functions
# with the structure of submodules/gsplat/cuda/_wrapper.py:573-1050 and the
# call sequence of scene/beta_model.py:660-722 + rendering.py:17-232.
class RefPipeline:
    def __init__(self, kernels=None):
        self.k = kernels or RefKernels()
        k = self.k

        class Rot(torch.autograd.Function):
            @staticmethod
            def forward(ctx, l3):
                return k.rotmat_fwd(l3.contiguous())

            @staticmethod
            def backward(ctx, vR):
                return k.rotmat_bwd(vR.contiguous())

        class Covar(torch.autograd.Function):
            @staticmethod
            def forward(ctx, R, s, l, ri, rj):
                ctx.save_for_backward(R, s, l, ri, rj)
                return k.covar_fwd(R.contiguous(), s.contiguous(), l.contiguous(), ri, rj)

            @staticmethod
            def backward(ctx, v):
                R, s, l, ri, rj = ctx.saved_tensors
                vr, vs, vl = k.covar_bwd(R, s, l, ri, rj, v.contiguous())
                return vr, vs, vl, None, None

        class Cond(torch.autograd.Function):
            @staticmethod
            def forward(ctx, m, V, o, b, q):
                args = [t.contiguous() for t in (m, V, o, b, q)]
                ctx.save_for_backward(*args)
                return k.cond_fwd(*args)

            @staticmethod
            def backward(ctx, vm, vV, vo):
                gm, gV, go, gb = k.cond_bwd(*ctx.saved_tensors, vm.contiguous(), vV.contiguous(),
                                            vo.contiguous())
                return gm, gV, go, gb, None

        class Proj(torch.autograd.Function):
            @staticmethod
            def forward(ctx, means, c6, vms, Ks, W, H):
                means, c6 = means.contiguous(), c6.contiguous()
                radii, m2, d, cn, _ = k.projection_fwd(means, c6, vms, Ks, W, H)
                ctx.save_for_backward(means, c6, vms, Ks, radii, cn)
                ctx.W, ctx.H = W, H
                ctx.mark_non_differentiable(radii)
                return radii, m2, d, cn

            @staticmethod
            def backward(ctx, vr, vm2, vd, vcn):
                means, c6, vms, Ks, radii, cn = ctx.saved_tensors
                C, N = radii.shape

                def z(t, *shape):
                    return torch.zeros(*shape, device=cn.device) if t is None else t.contiguous()
                vmeans, vcov, _ = k.projection_bwd(means, c6, vms, Ks, ctx.W, ctx.H, 0.3, radii, cn,
                                                   z(vm2, C, N, 2), z(vd, C, N), z(vcn, C, N, 3))
                return vmeans, vcov, None, None, None, None

        class Raster(torch.autograd.Function):
            @staticmethod
            def forward(ctx, m2, cn, col, op, be, bg, W, H, ts, offs, fl):
                args = [t.contiguous() for t in (m2, cn, col, op, be)]
                oc, oa, li = k.raster_fwd(*args, bg, W, H, ts, offs, fl)
                ctx.save_for_backward(*args, bg, offs, fl, oa, li)
                ctx.W, ctx.H, ctx.ts = W, H, ts
                return oc, oa

            @staticmethod
            def backward(ctx, vc, va):
                m2, cn, col, op, be, bg, offs, fl, oa, li = ctx.saved_tensors
                g = k.raster_bwd(m2, cn, col, op, be, bg, ctx.W, ctx.H, ctx.ts, offs, fl, oa, li,
                                 vc.contiguous(), va.contiguous())
                return g + (None,) * 6

        self.Rot, self.Covar, self.Cond, self.Proj, self.Raster = Rot, Covar, Cond, Proj, Raster

    def render_view(self, p, viewmat, K, W, H, center, background, rest_i, rest_j, tile_size=16,
                    timestamp=0.0):
        """Same operator sequence as the reference model's render + rasterization()
        (scene/beta_model.py:660-722): 6-D query = view direction, 7-D adds the
        timestamp."""
        import torch.nn.functional as F
        scale = F.softplus(p["scale"])
        beta = 4.0 * torch.exp(p["beta"])
        view_dir = p["xyz"] - center.unsqueeze(0)
        query = view_dir / view_dir.norm(dim=-1, keepdim=True)
        if p["scale"].shape[1] == 7:
            query = torch.cat([query, torch.full_like(query[:, :1], float(timestamp))], -1)
        R = self.Rot.apply(p["l_triangle"][:, :3])
        covar = self.Covar.apply(R, scale, p["l_triangle"], rest_i, rest_j)
        means_nd = torch.cat([p["xyz"], p["mean"]], -1)
        opac = torch.sigmoid(p["opacity"])
        means, convs, opacities = self.Cond.apply(means_nd, covar, opac, beta[:, 1:], query)
        c6 = convs[..., [0, 0, 0, 1, 1, 2], [0, 1, 2, 1, 2, 2]]
        vms, Ks = viewmat.unsqueeze(0), K.unsqueeze(0)
        radii, m2, d, cn = self.Proj.apply(means, c6, vms, Ks, W, H)
        op = opacities.squeeze(-1).repeat(1, 1)
        be = beta[:, 0].repeat(1, 1)
        tw, th = math.ceil(W / tile_size), math.ceil(H / tile_size)
        with torch.no_grad():
            _, ids, fl = self.k.isect_tiles(m2.detach(), radii, d.detach(), tile_size, tw, th)
            offs = self.k.offset_encode(ids, 1, tw, th)
        colors = p["rgb"].expand(1, -1, -1)
        oc, oa = self.Raster.apply(m2, cn, colors, op, be, background.unsqueeze(0), W, H,
                                   tile_size, offs, fl)
        return oc.permute(0, 3, 1, 2)[0], oa, dict(radii=radii, isect_ids=ids, flatten_ids=fl,
                                                   isect_offsets=offs[0])
