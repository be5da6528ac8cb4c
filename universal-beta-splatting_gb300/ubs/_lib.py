"""ctypes binding of the C ABI declared in include/ubs.h.

The library is the only compute path: there is no CPU or PyTorch fallback.
If it cannot be built or loaded, or a CUDA device is missing, calls raise.
"""
import ctypes
import os
import threading

import torch

from . import build as _build

_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_F = ctypes.c_float
_D = ctypes.c_double
_SZ = ctypes.c_size_t
_U32P = ctypes.POINTER(ctypes.c_uint32)
_I64P = ctypes.POINTER(ctypes.c_int64)
_INT = ctypes.c_int

# name -> (argtypes, restype); keep in step with include/ubs.h
SIGNATURES = {
    "ubs_last_error": ([], ctypes.c_char_p),
    "ubs_abi_version": ([], _INT),
    "ubs_l_triangle_to_rotmat_fwd": ([_I64, _P, _I64, _P, _P], _INT),
    "ubs_l_triangle_to_rotmat_bwd": ([_I64, _P, _P, _P], _INT),
    "ubs_rot_scale_l_triangle_to_covar_fwd": ([_I64, _I32, _P, _P, _P, _P, _P, _I32, _I32, _P, _P],
                                              _INT),
    "ubs_rot_scale_l_triangle_to_covar_bwd": ([_I64, _I32, _P, _P, _P, _P, _P, _I32, _I32, _P,
                                               _P, _P, _P, _P], _INT),
    "ubs_cond_fwd": ([_I64, _I32] + [_P] * 8 + [_P], _INT),
    "ubs_cond_bwd": ([_I64, _I32] + [_P] * 12 + [_I32, _P], _INT),
    "ubs_projection_fwd": ([_I32, _I64, _P, _P, _I32, _P, _P, _P, _P, _I32, _I32, _F, _F, _F, _F,
                            _P, _P, _P, _P, _P, _P], _INT),
    "ubs_projection_bwd": ([_I32, _I64, _P, _P, _I32, _P, _P, _P, _P, _I32, _I32, _F]
                           + [_P] * 7 + [_P] * 5 + [_P], _INT),
    "ubs_isect_count_workspace_bytes": ([_I32, _I64, _I32], _SZ),
    "ubs_isect_sort_workspace_bytes": ([_I32, _I64, _I32, _I64], _SZ),
    "ubs_isect_count": ([_I32, _I64, _P, _P, _P, _I32, _I32, _I32, _P, _P, _I64P, _P, _SZ, _P],
                        _INT),
    "ubs_isect_emit": ([_I32, _I64, _P, _P, _P, _I32, _I32, _I32, _P, _P, _I64, _I32, _P, _P, _P,
                        _SZ, _P], _INT),
    "ubs_isect_offset_encode": ([_I64, _P, _I32, _I32, _I32, _P, _P], _INT),
    "ubs_raster_workspace_bytes": ([_I64, _I32], _SZ),
    "ubs_raster_fwd": ([_I32, _I64, _I32, _I64] + [_P] * 7 + [_I32] * 5 + [_P] * 5 + [_P, _SZ, _P],
                       _INT),
    "ubs_raster_bwd": ([_I32, _I64, _I32, _I64] + [_P] * 7 + [_I32] * 5 + [_P] * 2 + [_P] * 4
                       + [_P] * 5 + [_P, _SZ, _P], _INT),
    "ubs_raster_pack": ([_I32, _I64, _I32, _I64] + [_P] * 6 + [_P, _SZ, _P], _INT),
    "ubs_raster_fwd_packed": ([_I32, _I64, _I32, _I64] + [_P] * 3 + [_I32] * 5 + [_P] * 4
                              + [_I32, _P, _SZ, _P], _INT),
    "ubs_raster_bwd_packed": ([_I32, _I64, _I32, _I64] + [_P] * 3 + [_I32] * 5 + [_P] * 3
                              + [_P] * 2 + [_P] * 5 + [_I32, _P, _SZ, _P], _INT),
    "ubs_raster_fwd_noalloc": ([_I32, _I64, _I32, _I64] + [_P] * 7 + [_I32] * 5 + [_P] * 5 + [_P],
                               _INT),
    "ubs_raster_status": ([_P, _U32P, ctypes.POINTER(ctypes.c_uint64), _P], _INT),
    "ubs_raster_noalloc_status": ([_U32P, _P], _INT),
    "ubs_set_blend_variant": ([_I32, _I32], _INT),
    "ubs_get_blend_variant": ([ctypes.POINTER(_I32), ctypes.POINTER(_I32)], _INT),
    "ubs_launch_count": ([], ctypes.c_ulonglong),
    "ubs_scene_workspace_bytes": ([_I32, _I64, _I32, _I64], _SZ),
    "ubs_scene_forward": ([_I32, _I64] + [_P] * 7 + [_I32] + [_P] * 7 + [_I32, _I32, _F, _F, _F, _F]
                          + [_P] * 4 + [_I64, _P, _SZ, _P], _INT),
    "ubs_raster_pair_counts": ([_P, _P, _P], _INT),
    "ubs_scene_workspace_offsets": ([_I32, _I64, _I32, _I64, _I64P, _I64P], _INT),
    "ubs_scene_workspace_layout": ([_I32, _I64, _I32, _I64, _I64P, _I32], _INT),
    "ubs_scene_forward_masked": ([_I32, _I64] + [_P] * 7 + [_I32] + [_P] * 7
                                 + [_I32, _I32, _F, _F, _F, _F] + [_P] * 4
                                 + [_I64, _P, _SZ, _P, _I32, _P], _INT),
    "ubs_scene_backward": ([_I32, _I64] + [_P] * 7 + [_I32] + [_P] * 7 + [_I32, _I32, _F, _F, _F, _F]
                           + [_P] * 5 + [_P] * 7 + [_I32, _I64, _P, _SZ, _P], _INT),
    "ubs_scene_stats": ([_P, _I64P, _U32P, _P], _INT),
    "ubs_profile_start": ([_I32], _INT),
    "ubs_profile_stop": ([ctypes.POINTER(_I32)], _INT),
    "ubs_profile_sample": ([], _INT),
    "ubs_profile_result": ([_I32, ctypes.POINTER(ctypes.c_char_p), _I64P,
                            ctypes.POINTER(ctypes.c_double)], _INT),
    "ubs_adam_table_bytes": ([_I32], _SZ),
    "ubs_adam_table_entry": ([_P, _I32, _P, _P, _P, _P, _I64, _I32], _INT),
    "ubs_adam_step": ([_I32, _P, _P, _I64, _I64, _F, _F, _F, _F, _P], _INT),
    "ubs_quantile_mask_workspace_bytes": ([], _SZ),
    "ubs_quantile_mask": ([_I64, _I32, _P, _P, _P, _P, _P, _SZ, _P], _INT),
    "ubs_quantile_mask_bounds": ([_P, _I32, _P, _P], _INT),
    "ubs_depth_colormap": ([_P, _I64, _P, _P, _P, _P], _INT),
    "ubs_ply_read_header": ([ctypes.c_char_p, _I64P, ctypes.POINTER(ctypes.c_int32), _P, _I32,
                             _I64P], _INT),
    "ubs_ply_read_body": ([ctypes.c_char_p, _I64, _P, _I64], _INT),
    "ubs_ply_write": ([ctypes.c_char_p, _I64, _I32, _P, _P], _INT),
    "ubs_ply_unpack": ([_P, _P, _I64, _P], _INT),
    "ubs_ply_pack": ([_P, _P, _I64, _P], _INT),
    "ubs_mcmc_workspace_bytes": ([_I64, _I64], _SZ),
    "ubs_mcmc_relocate": ([_P, _I64, _P, _F, ctypes.c_uint64, _P, _I64, _P, _P, _SZ, _P], _INT),
    "ubs_mcmc_add": ([_P, _P, _I64, _I64, ctypes.c_uint64, _P, _P, _P, _SZ, _P], _INT),
    "ubs_mcmc_perturb_xyz": ([_I64, _I32, _P, _P, _P, _P, _F, ctypes.c_uint64, _P, _P], _INT),
    "ubs_ssim_workspace_bytes": ([_I32, _I32, _I32, _I32], _SZ),
    "ubs_l1_loss_workspace_bytes": ([_I64], _SZ),
    "ubs_l1_loss": ([_P, _P, _P, _I64, _D, _P, _P, _SZ, _P], _INT),
    "ubs_ssim_loss": ([_P, _P, _P, _P, _P, _P, _I32, _I32, _I32, _I32, _I32, _D, _D, _D, _P,
                       _P, _SZ, _P], _INT),
    "ubs_fp32_probe_workspace_bytes": ([], _SZ),
    "ubs_fp32_probe": ([_I32, _P, _SZ, ctypes.POINTER(ctypes.c_double), _P], _INT),
    "ubs_mufu_probe": ([_I32, _P, _SZ, ctypes.POINTER(ctypes.c_double), _P], _INT),
}

_lib = None
_lock = threading.Lock()


def lib():
    """Load (building first if needed) the native library."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                path = _build.build()
                L = ctypes.CDLL(path)
                for name, (argt, rest) in SIGNATURES.items():
                    fn = getattr(L, name)
                    fn.argtypes = argt
                    fn.restype = rest
                _lib = L
    return _lib


def library_path():
    return _build.LIB_PATH


def last_error():
    return lib().ubs_last_error().decode(errors="replace")


_timing = None  # list of (name, start_event, end_event) while timing is on


def call(name, *args):
    """Call an int-returning entry point and raise on a non-zero status."""
    if _timing is not None:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        rc = getattr(lib(), name)(*args)
        e1.record()
        _timing.append((name, e0, e1))
    else:
        rc = getattr(lib(), name)(*args)
    if rc != 0:
        raise RuntimeError("%s failed (%d): %s" % (name, rc, last_error()))
    return rc


def start_timing():
    """Record CUDA events (on the current stream) around every entry-point call."""
    global _timing
    _timing = []


def stop_timing():
    """Stop recording; returns {entry point: (calls, total ms)}."""
    global _timing
    rec, _timing = _timing or [], None
    torch.cuda.synchronize()
    out = {}
    for name, e0, e1 in rec:
        n, t = out.get(name, (0, 0.0))
        out[name] = (n + 1, t + e0.elapsed_time(e1))
    return out


def profile_start(max_launches=4096):
    """Time every kernel the library launches from now on (CUDA events on the
    launching stream)."""
    call("ubs_profile_start", int(max_launches))


def profile_sample():
    """After a CUDA-graph replay: add the replay's kernel durations."""
    call("ubs_profile_sample")


def profile_stop():
    """Stop kernel timing; returns {kernel: (launches, total ms)}."""
    n = ctypes.c_int32(0)
    call("ubs_profile_stop", ctypes.byref(n))
    out = {}
    for i in range(n.value):
        name, cnt, ms = ctypes.c_char_p(), ctypes.c_int64(), ctypes.c_double()
        call("ubs_profile_result", i, ctypes.byref(name), ctypes.byref(cnt), ctypes.byref(ms))
        out[name.value.decode()] = (int(cnt.value), float(ms.value))
    return out


def query(name, *args):
    return getattr(lib(), name)(*args)


def ptr(t, dtype=None):
    """Device pointer of a contiguous CUDA tensor (None passes NULL)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor, got device %s" % t.device)
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    if dtype is not None and t.dtype != dtype:
        raise TypeError("expected dtype %s, got %s" % (dtype, t.dtype))
    return ctypes.c_void_p(t.data_ptr())


def strided_ptr(t):
    """Device pointer of a CUDA tensor whose strides the callee is given."""
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor, got device %s" % t.device)
    return ctypes.c_void_p(t.data_ptr())


def stream(device=None):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def stream_ptr(s):
    """cudaStream_t of a torch.cuda.Stream."""
    return ctypes.c_void_p(s.cuda_stream)


def workspace(nbytes, device):
    """Caller-owned scratch memory (the caching allocator aligns to 512 bytes)."""
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
