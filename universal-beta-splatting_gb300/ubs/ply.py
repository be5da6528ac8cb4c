"""Scene files: the reference's PLY format, loaded straight into device memory.

The reference saves a scene as one PLY vertex element of float32 properties in
the order x, y, z, red, green, blue, opacity, beta_*, mean_*, scale_*,
l_triangle_* (scene/beta_model.py:286-320) and loads it back by property name,
sorting each family by its numeric suffix (:322-404).  Here the header is
parsed and the body read by the library's host code into pinned memory in
chunks, each chunk's copy to the device overlapping the next chunk's read, and
one kernel scatters the records into the seven parameter tensors; saving runs
the inverse (one gather kernel, one copy to the host, one write).

    load_ply(path, device)           -> dict of raw parameter tensors
    save_ply(path, params)
    load_model_ply(model, path)      BetaModel.load_ply drop-in (nn.Parameters)
    save_model_ply(model, path)      BetaModel.save_ply drop-in
"""
import ctypes
import math
import os

import torch

from . import _lib as L

NAMES = ("xyz", "mean", "rgb", "opacity", "beta", "scale", "l_triangle")
MAX_TENSORS, MAX_PROPS, NAME_BYTES = 8, 256, 64
CHUNK_BYTES = 64 << 20


class _Layout(ctypes.Structure):
    _fields_ = [("record_floats", ctypes.c_int32), ("n_tensors", ctypes.c_int32),
                ("width", ctypes.c_int32 * MAX_TENSORS),
                ("param", ctypes.c_void_p * MAX_TENSORS),
                ("tensor_of", ctypes.c_int16 * MAX_PROPS),
                ("column_of", ctypes.c_int16 * MAX_PROPS)]


def attribute_names(widths):
    """Property names in the reference's order (construct_list_of_attributes,
    scene/beta_model.py:286-296) for tensor widths {name: width}."""
    names = ["x", "y", "z", "red", "green", "blue", "opacity"]
    names += ["beta_%d" % i for i in range(widths["beta"])]
    names += ["mean_%d" % i for i in range(widths["mean"])]
    names += ["scale_%d" % i for i in range(widths["scale"])]
    names += ["l_triangle_%d" % i for i in range(widths["l_triangle"])]
    return names


def _family(names, prefix):
    """Indices of the properties named prefix*, sorted by their numeric suffix
    (how the reference's load_ply orders each family)."""
    idx = [i for i, n in enumerate(names) if n.startswith(prefix)]
    return sorted(idx, key=lambda i: int(names[i].split("_")[-1]))


def column_map(names):
    """{tensor: [property index of each column]} as the reference's load_ply
    reads them; raises KeyError where it would."""
    pos = {n: i for i, n in enumerate(names)}
    return {"xyz": [pos["x"], pos["y"], pos["z"]],
            "rgb": [pos["red"], pos["green"], pos["blue"]],
            "opacity": [pos["opacity"]],
            "mean": _family(names, "mean_"),
            "beta": _family(names, "beta_"),
            "scale": _family(names, "scale_"),
            "l_triangle": _family(names, "l_triangle")}


def _layout(n_props, cmap, tensors):
    lay = _Layout()
    lay.record_floats = n_props
    lay.n_tensors = len(NAMES)
    for c in range(MAX_PROPS):
        lay.tensor_of[c] = -1
        lay.column_of[c] = 0
    for k, name in enumerate(NAMES):
        t = tensors[name]
        lay.width[k] = t.shape[1]
        lay.param[k] = t.data_ptr()
        for j, c in enumerate(cmap[name]):
            lay.tensor_of[c] = k
            lay.column_of[c] = j
    return lay


def read_header(path):
    """(vertex count, property names, body offset)."""
    nv, npr, off = ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int64()
    bpath = os.fsencode(path)
    L.call("ubs_ply_read_header", bpath, ctypes.byref(nv), ctypes.byref(npr), None, 0,
           ctypes.byref(off))
    buf = ctypes.create_string_buffer(npr.value * NAME_BYTES)
    L.call("ubs_ply_read_header", bpath, ctypes.byref(nv), ctypes.byref(npr), buf, npr.value,
           ctypes.byref(off))
    names = [buf.raw[i * NAME_BYTES:(i + 1) * NAME_BYTES].split(b"\0", 1)[0].decode()
             for i in range(npr.value)]
    return nv.value, names, off.value


@torch.no_grad()
def load_ply(path, device="cuda"):
    """The scene in `path` as raw parameter tensors on `device`."""
    n, names, off = read_header(path)
    cmap = column_map(names)
    A = len(names)
    dev = torch.device(device)
    out = {k: torch.empty(n, len(cmap[k]), dtype=torch.float32, device=dev) for k in NAMES}
    if n == 0:
        return out
    total = n * A * 4
    records = torch.empty(n * A, dtype=torch.float32, device=dev)
    rec_bytes = records.view(torch.uint8)
    chunk = max(A * 4, (CHUNK_BYTES // (A * 4)) * A * 4)
    bufs = [torch.empty(min(chunk, total), dtype=torch.uint8, pin_memory=True)
            for _ in range(2)]
    events = [None, None]
    bpath = os.fsencode(path)
    stream = torch.cuda.current_stream(dev)
    done, i = 0, 0
    while done < total:
        nb = min(chunk, total - done)
        buf = bufs[i & 1]
        if events[i & 1] is not None:
            events[i & 1].synchronize()  # the copy that last read this buffer is done
        L.call("ubs_ply_read_body", bpath, off + done, ctypes.c_void_p(buf.data_ptr()), nb)
        rec_bytes[done:done + nb].copy_(buf[:nb], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(stream)
        events[i & 1] = ev
        done += nb
        i += 1
    lay = _layout(A, cmap, out)
    L.call("ubs_ply_unpack", ctypes.byref(lay), L.ptr(records), n, L.stream(dev))
    for ev in events:  # keep the pinned buffers alive until their copies end
        if ev is not None:
            ev.synchronize()
    return out


@torch.no_grad()
def save_ply(path, params):
    """Write raw parameter tensors (the reference's names) as its PLY file."""
    t = {}
    for k in NAMES:
        v = params[k].detach()
        t[k] = v.reshape(v.shape[0], int(math.prod(v.shape[1:]))).contiguous()
    n = t["xyz"].shape[0]
    dev = t["xyz"].device
    if not t["xyz"].is_cuda:
        raise TypeError("save_ply packs on the device: pass CUDA tensors")
    names = attribute_names({k: v.shape[1] for k, v in t.items()})
    A = len(names)
    cmap = column_map(names)
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    records = torch.empty(max(1, n * A), dtype=torch.float32, device=dev)
    lay = _layout(A, cmap, t)
    L.call("ubs_ply_pack", ctypes.byref(lay), L.ptr(records), n, L.stream(dev))
    host = torch.empty(max(1, n * A), dtype=torch.float32, pin_memory=True)
    host.copy_(records, non_blocking=True)
    torch.cuda.current_stream(dev).synchronize()
    nbuf = ctypes.create_string_buffer(A * NAME_BYTES)
    for i, nm in enumerate(names):
        raw = nm.encode()[:NAME_BYTES - 1]
        ctypes.memmove(ctypes.addressof(nbuf) + i * NAME_BYTES, raw, len(raw))
    L.call("ubs_ply_write", os.fsencode(path), n, A, nbuf, ctypes.c_void_p(host.data_ptr()))


def load_model_ply(model, path, device="cuda"):
    """BetaModel.load_ply: the file's tensors become the model's parameters."""
    p = load_ply(path, device)
    for k in NAMES:
        setattr(model, "_" + k, torch.nn.Parameter(p[k].requires_grad_(True)))


def save_model_ply(model, path):
    """BetaModel.save_ply."""
    save_ply(path, {k: getattr(model, "_" + k) for k in NAMES})
