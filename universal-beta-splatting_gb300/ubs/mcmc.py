"""MCMC densification on the device (csrc/mcmc.cu).

Drop-in functions for the reference's BetaModel methods and the noise step of
its training loop, operating on any object with the BetaModel attributes
(`_xyz, _mean, _rgb, _opacity, _beta, _scale, _l_triangle` and `optimizer`):

    relocate_gs(model, dead_mask)   scene/beta_model.py:585-621
    add_new_gs(model, cap_max)      scene/beta_model.py:623-658
    perturb_xyz(model, factor)      train.py:164-171 (factor = noise_lr * xyz_lr)

The reference synchronises with the device several times per call (mask sums,
nonzero, multinomial); these launch a fixed sequence of kernels and never
wait.  The draws come from the library's counter-based generator seeded from
torch's CPU generator, so they are reproducible under torch.manual_seed but are
not torch.multinomial's; `src=` takes given draws (one source index per dead
or new primitive) and then reproduces the reference exactly.  Optimizer state
(torch.optim.Adam or ubs.optim.FusedAdam, keys exp_avg / exp_avg_sq) is edited
as the reference edits it; add_new_gs re-registers the grown parameters in the
optimizer's groups under their names.
"""
import ctypes
import math

import torch

from . import _lib as L

NAMES = ("xyz", "mean", "rgb", "opacity", "beta", "scale", "l_triangle")
MAX_TENSORS = 8
DEAD_OPACITY = 0.005  # train.py:161


class _Tensors(ctypes.Structure):
    _fields_ = [("n_tensors", ctypes.c_int32), ("opacity_index", ctypes.c_int32),
                ("width", ctypes.c_int32 * MAX_TENSORS),
                ("param", ctypes.c_void_p * MAX_TENSORS),
                ("exp_avg", ctypes.c_void_p * MAX_TENSORS),
                ("exp_avg_sq", ctypes.c_void_p * MAX_TENSORS)]


def _seed(generator):
    return int(torch.randint(0, 2 ** 62, (1,), generator=generator).item())


def _params(model):
    return [getattr(model, "_" + k) for k in NAMES]


def _state(optimizer, p):
    if optimizer is None:
        return None
    st = optimizer.state.get(p)
    if not st or "exp_avg" not in st:
        return None
    return st


def _check(tensors):
    n = tensors[0].shape[0]
    for t in tensors:
        if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
            raise TypeError("MCMC tensors must be contiguous float32 CUDA tensors")
        if t.shape[0] != n:
            raise ValueError("MCMC tensors must have one row per primitive")
    return n


def _set(params, moments):
    s = _Tensors()
    s.n_tensors = len(params)
    s.opacity_index = NAMES.index("opacity")
    for k, p in enumerate(params):
        s.width[k] = int(math.prod(p.shape[1:]))
        s.param[k] = p.data_ptr()
        m, v = moments[k]
        s.exp_avg[k] = m.data_ptr() if m is not None else None
        s.exp_avg_sq[k] = v.data_ptr() if v is not None else None
    return s


def _moments(optimizer, params):
    out = []
    for p in params:
        st = _state(optimizer, p)
        out.append((st["exp_avg"], st["exp_avg_sq"]) if st is not None else (None, None))
    for m, v in out:
        if m is not None:
            _check([m, v])
    return out


def _status(dev):
    return torch.zeros(1, dtype=torch.int32, device=dev)


@torch.no_grad()
def relocate_gs(model, dead_mask=None, generator=None, src=None, status=None):
    """Move the dead primitives (dead_mask, default sigmoid(opacity) <= 0.005)
    onto opacity-sampled live ones, in place.  `status` (int32 device tensor)
    receives error bits for bad given draws."""
    params = _params(model)
    n = _check(params)
    if n == 0:
        return
    dev = params[0].device
    moments = _moments(model.optimizer, params)
    s = _set(params, moments)
    mask = None
    if dead_mask is not None:
        mask = dead_mask.reshape(-1)
        if mask.shape[0] != n:
            raise ValueError("dead_mask needs one entry per primitive")
        mask = mask.to(torch.uint8).contiguous()
    given = None
    if src is not None:
        given = src.to(device=dev, dtype=torch.int64).contiguous()
    ws = L.workspace(L.query("ubs_mcmc_workspace_bytes", n, n), dev)
    st = status if status is not None else _status(dev)
    L.call("ubs_mcmc_relocate", ctypes.byref(s), n, L.ptr(mask), DEAD_OPACITY,
           _seed(generator) if given is None else 0, L.ptr(given),
           0 if given is None else given.numel(), L.ptr(st), L.ptr(ws), ws.numel(),
           L.stream(dev))
    return st


@torch.no_grad()
def add_new_gs(model, cap_max, generator=None, src=None, status=None):
    """Append min(cap_max, int(1.02 n)) - n opacity-sampled copies; returns how
    many (known on the host: no synchronisation).  The model's parameters are
    replaced by the grown tensors, in the optimizer too."""
    params = _params(model)
    n = _check(params)
    n_add = max(0, min(int(cap_max), int(1.02 * n)) - n)
    if n_add <= 0 or n == 0:
        return 0
    dev = params[0].device
    opt = model.optimizer
    moments = _moments(opt, params)
    grown = [torch.empty((n + n_add,) + tuple(p.shape[1:]), dtype=p.dtype, device=dev)
             for p in params]
    grown_m = [(torch.empty_like(g), torch.empty_like(g)) if m is not None else (None, None)
               for g, (m, _) in zip(grown, moments)]
    given = None
    if src is not None:
        given = src.to(device=dev, dtype=torch.int64).contiguous()
        if given.numel() != n_add:
            raise ValueError("src needs one index per new primitive (%d)" % n_add)
    ws = L.workspace(L.query("ubs_mcmc_workspace_bytes", n, n_add), dev)
    st = status if status is not None else _status(dev)
    s_old, s_new = _set(params, moments), _set(grown, grown_m)
    L.call("ubs_mcmc_add", ctypes.byref(s_old), ctypes.byref(s_new), n, n_add,
           _seed(generator) if given is None else 0, L.ptr(given), L.ptr(st), L.ptr(ws),
           ws.numel(), L.stream(dev))
    # re-register, as cat_tensors_to_optimizer / replace_tensors_to_optimizer do
    for name, old, new, (m, v) in zip(NAMES, params, grown, grown_m):
        p = torch.nn.Parameter(new.requires_grad_(True))
        if opt is not None:
            for group in opt.param_groups:
                if group["params"] and group["params"][0] is old:
                    group["params"][0] = p
            stv = opt.state.pop(old, None)
            if stv is not None:
                if m is not None:
                    stv["exp_avg"], stv["exp_avg_sq"] = m, v
                opt.state[p] = stv
        setattr(model, "_" + name, p)
    return n_add


@torch.no_grad()
def perturb_xyz(model, factor, generator=None, noise=None):
    """xyz += Sigma_xyz (z (1 - opacity)^100 factor), z ~ N(0, I) (or `noise`)."""
    xyz, op, sc, lt = model._xyz, model._opacity, model._scale, model._l_triangle
    n = _check([xyz, op, sc, lt])
    if n == 0:
        return
    dim = sc.shape[1]
    if noise is not None:
        noise = noise.to(device=xyz.device, dtype=torch.float32).contiguous()
    L.call("ubs_mcmc_perturb_xyz", n, dim, L.ptr(xyz), L.ptr(op), L.ptr(sc), L.ptr(lt),
           float(factor), _seed(generator) if noise is None else 0, L.ptr(noise),
           L.stream(xyz.device))
